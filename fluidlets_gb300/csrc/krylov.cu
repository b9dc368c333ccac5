// krylov.cu -- restarted GMRES and GMRES-based iterative refinement.
//
// flg_gmres replaces the GMRES branch of fluidlets.resistance
// (core/solve.py:68-79), which calls scipy.sparse.linalg.gmres with
// rtol, atol = 0, restart, maxiter and a "pr_norm" callback counting inner
// iterations.  The outer structure below follows SciPy's implementation
// (scipy/sparse/linalg/_isolve/iterative.py, gmres): restart cycles,
// Givens rotations with LAPACK lartg conventions, the true residual
// recomputed after every cycle, and the adaptive inner tolerance of
// gh-8400.  Orthogonalization is classical Gram-Schmidt with one
// re-orthogonalization (CGS2), so each inner iteration costs two
// multi-vector dot products and two multi-vector updates on the device and
// a single device-to-host copy of the new Hessenberg column.
//
// The iterative refinements (mixed-precision flg_gmres, flg_gmres_ir_dense)
// pass their inner solves the known ||r|| and a zero start, which saves three
// host round trips per inner solve without changing the arithmetic.
//
// Dot products are deterministic: fixed chunking, per-chunk block
// reductions, then an in-order sum of the chunk partials.
#include <algorithm>
#include <cmath>
#include <complex>
#include <functional>
#include <vector>

#include "flg_common.cuh"
#include "sum_plan.cuh"

namespace flg {

using cplx_h = std::complex<double>;

// ---- scalar traits: double (real) or double2 (complex) ----------------------
template <typename T>
struct S;
template <>
struct S<double> {
    using H = double;
    static constexpr bool complex = false;
    __device__ static double zero() { return 0.0; }
    __device__ static double conj_mul(double a, double b) { return a * b; }
    __device__ static double mul(double a, double b) { return a * b; }
    __device__ static double add(double a, double b) { return a + b; }
    __device__ static double sub(double a, double b) { return a - b; }
    __device__ static double shfl(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
    static H to_h(double v) { return v; }
    static double from_h(H v) { return v; }
};
template <>
struct S<double2> {
    using H = cplx_h;
    static constexpr bool complex = true;
    __device__ static double2 zero() { return make_double2(0.0, 0.0); }
    __device__ static double2 conj_mul(double2 a, double2 b) {  // conj(a) * b
        return make_double2(fma(a.x, b.x, a.y * b.y), fma(a.x, b.y, -a.y * b.x));
    }
    __device__ static double2 mul(double2 a, double2 b) {
        return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
    }
    __device__ static double2 add(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
    __device__ static double2 sub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
    __device__ static double2 shfl(double2 v, int o) {
        return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
    }
    static H to_h(double2 v) { return H(v.x, v.y); }
    static double2 from_h(H v) { return make_double2(v.real(), v.imag()); }
};

constexpr int kDotThreads = 256;
constexpr int64_t kDotChunk = 8192;  // elements per CTA and vector

// partial[k * nchunk + c] = sum_{i in chunk c} conj(V[k][i]) w[i]
template <typename T>
__global__ void __launch_bounds__(kDotThreads) dot_partial_kernel(const T *V, int64_t ldv, const T *w, int64_t n,
                                                                  int64_t nchunk, T *partial) {
    __shared__ T sm[kDotThreads / 32];
    const int k = blockIdx.y;
    const int64_t c = blockIdx.x;
    const T *v = V + (int64_t)k * ldv;
    T acc = S<T>::zero();
    const int64_t lo = c * kDotChunk, hi = min(n, lo + kDotChunk);
    for (int64_t i = lo + threadIdx.x; i < hi; i += kDotThreads) acc = S<T>::add(acc, S<T>::conj_mul(v[i], w[i]));
    for (int o = 16; o > 0; o >>= 1) acc = S<T>::add(acc, S<T>::shfl(acc, o));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        T s = S<T>::zero();
        for (int q = 0; q < kDotThreads / 32; q++) s = S<T>::add(s, sm[q]);
        partial[(int64_t)k * nchunk + c] = s;
    }
}

template <typename T>
__global__ void dot_finish_kernel(const T *partial, int64_t nchunk, int nvec, T *out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nvec) return;
    T s = S<T>::zero();
    for (int64_t c = 0; c < nchunk; c++) s = S<T>::add(s, partial[(int64_t)k * nchunk + c]);
    out[k] = s;
}

// w -= sum_k V[k] h[k]
template <typename T>
__global__ void gemv_sub_kernel(const T *V, int64_t ldv, int nvec, const T *h, T *w, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = w[i];
    for (int k = 0; k < nvec; k++) acc = S<T>::sub(acc, S<T>::mul(V[(int64_t)k * ldv + i], h[k]));
    w[i] = acc;
}

// x += sum_k V[k] y[k]  (y by value in a small device array)
template <typename T>
__global__ void gemv_add_kernel(const T *V, int64_t ldv, int nvec, const T *y, T *x, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    T acc = S<T>::zero();
    for (int k = 0; k < nvec; k++) acc = S<T>::add(acc, S<T>::mul(V[(int64_t)k * ldv + i], y[k]));
    x[i] = S<T>::add(x[i], acc);
}

template <typename T>
__global__ void scale_kernel(T *x, int64_t n, double s) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if constexpr (S<T>::complex) x[i] = make_double2(x[i].x * s, x[i].y * s);
    else x[i] = x[i] * s;
}

// y = a - y   (residual r = b - A x, with y = A x on input)
template <typename T>
__global__ void rsub_kernel(const T *a, T *y, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = S<T>::sub(a[i], y[i]);
}

template <typename T>
__global__ void add_kernel(T *x, const T *d, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = S<T>::add(x[i], d[i]);
}

__global__ void any_nonzero_kernel(const double *x, int64_t n, int *flag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && x[i] != 0.0) *flag = 1;
}

// ---- GMRES ---------------------------------------------------------------------
template <typename T>
struct Gmres {
    using H = typename S<T>::H;
    int64_t n = 0;
    int m = 0;
    cudaStream_t st = nullptr;
    T *V = nullptr;        // (m + 1) x n Krylov basis
    T *r = nullptr;        // residual
    T *tmp = nullptr;      // operator scratch
    T *partial = nullptr;  // dot partials: (m + 2) x nchunk
    T *hdev = nullptr;     // 3 (m + 2) scalars
    int *flag = nullptr;
    int64_t nchunk = 0;
    // y = A v ; y = M^-1 v (optional)
    std::function<int(const T *, T *)> A, M;

    static void carve_sizes(int64_t n, int m, CountingArena &c) {
        const int64_t nchunk = ceil_div(std::max<int64_t>(n, 1), kDotChunk);
        c.take<T>((size_t)(m + 1) * n);
        c.take<T>(n);
        c.take<T>(n);
        c.take<T>((size_t)(m + 2) * nchunk);
        c.take<T>(3 * (m + 2));
        c.take<int>(1);
    }
    bool carve(int64_t n_, int m_, Arena &ar) {
        n = n_;
        m = m_;
        nchunk = ceil_div(std::max<int64_t>(n, 1), kDotChunk);
        V = ar.take<T>((size_t)(m + 1) * n);
        r = ar.take<T>(n);
        tmp = ar.take<T>(n);
        partial = ar.take<T>((size_t)(m + 2) * nchunk);
        hdev = ar.take<T>(3 * (m + 2));
        flag = ar.take<int>(1);
        return V && r && tmp && partial && hdev && flag;
    }

    int grid(int64_t k) const { return (int)ceil_div(k, 256); }

    // out[0..nvec) = V[0..nvec)^H w (device)
    int dots(const T *Vb, int nvec, const T *w, T *out) {
        dim3 g((unsigned)nchunk, (unsigned)nvec);
        dot_partial_kernel<T><<<g, kDotThreads, 0, st>>>(Vb, n, w, n, nchunk, partial);
        FLG_LAUNCH_CHECK();
        dot_finish_kernel<T><<<(nvec + 63) / 64, 64, 0, st>>>(partial, nchunk, nvec, out);
        FLG_LAUNCH_CHECK();
        return FLG_OK;
    }
    int norm(const T *w, double *out) {
        T d;
        FLG_TRY(dots(w, 1, w, hdev));
        FLG_CUDA(cudaMemcpyAsync(&d, hdev, sizeof(T), cudaMemcpyDeviceToHost, st));
        FLG_CUDA(cudaStreamSynchronize(st));
        if constexpr (S<T>::complex) *out = std::sqrt(std::max(d.x, 0.0));
        else *out = std::sqrt(std::max(d, 0.0));
        return FLG_OK;
    }
    int apply(const T *v, T *out) {  // out = M^-1 A v
        if (!M) return A(v, out);
        FLG_TRY(A(v, tmp));
        return M(tmp, out);
    }
    int precond(const T *v, T *out) {
        if (!M) {
            FLG_CUDA(cudaMemcpyAsync(out, v, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
            return FLG_OK;
        }
        return M(v, out);
    }
    // r = b - A x
    int residual(const T *b, const T *x) {
        FLG_TRY(A(x, r));
        rsub_kernel<T><<<grid(n), 256, 0, st>>>(b, r, n);
        FLG_LAUNCH_CHECK();
        return FLG_OK;
    }

    // r = b - A x, or r = b without the operator when x is all zeros (the start of an
    // iterative refinement; the FP64 kernel sum that would give A 0 costs a full matvec);
    // *is_b tells which
    int residual_from(const T *b, const T *x, bool *is_b) {
        int nz = 0;
        FLG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
        any_nonzero_kernel<<<grid(n * (S<T>::complex ? 2 : 1)), 256, 0, st>>>((const double *)x,
                                                                             n * (S<T>::complex ? 2 : 1), flag);
        FLG_LAUNCH_CHECK();
        FLG_CUDA(cudaMemcpyAsync(&nz, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
        FLG_CUDA(cudaStreamSynchronize(st));
        *is_b = nz == 0;
        if (nz) return residual(b, x);
        FLG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
        return FLG_OK;
    }

    static void lartg(H f, H g, double &c, H &s, H &rr) {
        if constexpr (!S<T>::complex) {
            if (g == 0.0) {
                c = 1.0;
                s = 0.0;
                rr = f;
            } else if (f == 0.0) {
                c = 0.0;
                s = g > 0 ? 1.0 : -1.0;
                rr = std::fabs(g);
            } else {
                const double d = std::hypot(f, g);
                c = std::fabs(f) / d;
                rr = f > 0 ? d : -d;
                s = g / rr;
            }
        } else {
            if (g == H(0.0)) {
                c = 1.0;
                s = 0.0;
                rr = f;
            } else if (f == H(0.0)) {
                c = 0.0;
                const double ag = std::abs(g);
                s = std::conj(g) / ag;
                rr = ag;
            } else {
                const double af = std::abs(f), ag = std::abs(g);
                const double d = std::hypot(af, ag);
                c = af / d;
                const H ph = f / af;
                rr = ph * d;
                s = ph * std::conj(g) / d;
            }
        }
    }

    // host side of one restart cycle: Hessenberg, Givens rotations, least-squares solution
    struct Scratch {
        std::vector<H> h, S_, y, gs;
        std::vector<double> gc;
        std::vector<T> hbuf;
        explicit Scratch(int m)
            : h((size_t)m * (m + 1)), S_(m + 1), y(m + 1), gs(m), gc(m), hbuf(2 * (m + 2) + 2) {}
    };

    // One restart cycle from V[0] = v / beta (V[0] holds v on entry): Arnoldi with two
    // classical Gram-Schmidt passes and Givens rotations until the estimated residual
    // presid <= ptol, a breakdown, or m columns; then x += V y.  iters += columns.
    int cycle(T *x, double beta, double ptol, int &iters, double &presid, bool &breakdown, Scratch &hs) {
        const double eps = 2.220446049250313e-16;
        std::vector<H> &h = hs.h, &S_ = hs.S_, &y = hs.y, &gs = hs.gs;
        std::vector<double> &gc = hs.gc;
        std::vector<T> &hbuf = hs.hbuf;
        scale_kernel<T><<<grid(n), 256, 0, st>>>(V, n, 1.0 / beta);
        FLG_LAUNCH_CHECK();
        std::fill(S_.begin(), S_.end(), H(0.0));
        S_[0] = beta;
        breakdown = false;
        int col = 0;
        for (col = 0; col < m; col++) {
            T *w = V + (int64_t)(col + 1) * n;
            FLG_TRY(apply(V + (int64_t)col * n, w));
            // device: [h1 (col+1) | h2 (col+1) | |w|^2 before | |w|^2 after]
            T *h1d = hdev, *h2d = hdev + (col + 1), *nb = hdev + 2 * (col + 1), *na = nb + 1;
            FLG_TRY(dots(w, 1, w, nb));
            FLG_TRY(dots(V, col + 1, w, h1d));
            gemv_sub_kernel<T><<<grid(n), 256, 0, st>>>(V, n, col + 1, h1d, w, n);
            FLG_LAUNCH_CHECK();
            FLG_TRY(dots(V, col + 1, w, h2d));
            gemv_sub_kernel<T><<<grid(n), 256, 0, st>>>(V, n, col + 1, h2d, w, n);
            FLG_LAUNCH_CHECK();
            FLG_TRY(dots(w, 1, w, na));
            FLG_CUDA(cudaMemcpyAsync(hbuf.data(), hdev, sizeof(T) * (2 * (col + 1) + 2), cudaMemcpyDeviceToHost,
                                     st));
            FLG_CUDA(cudaStreamSynchronize(st));
            H *hc = &h[(size_t)col * (m + 1)];
            for (int k = 0; k <= col; k++) hc[k] = S<T>::to_h(hbuf[k]) + S<T>::to_h(hbuf[col + 1 + k]);
            double h0, h1n;
            if constexpr (S<T>::complex) {
                h0 = std::sqrt(std::max(hbuf[2 * (col + 1)].x, 0.0));
                h1n = std::sqrt(std::max(hbuf[2 * (col + 1) + 1].x, 0.0));
            } else {
                h0 = std::sqrt(std::max(hbuf[2 * (col + 1)], 0.0));
                h1n = std::sqrt(std::max(hbuf[2 * (col + 1) + 1], 0.0));
            }
            hc[col + 1] = h1n;
            if (h1n <= eps * h0) {
                hc[col + 1] = 0.0;
                breakdown = true;
            } else {
                scale_kernel<T><<<grid(n), 256, 0, st>>>(w, n, 1.0 / h1n);
                FLG_LAUNCH_CHECK();
            }
            for (int k = 0; k < col; k++) {
                const double c = gc[k];
                const H s = gs[k];
                const H n0 = hc[k], n1 = hc[k + 1];
                hc[k] = c * n0 + s * n1;
                if constexpr (S<T>::complex) hc[k + 1] = -std::conj(s) * n0 + c * n1;
                else hc[k + 1] = -s * n0 + c * n1;
            }
            double c;
            H s, mag;
            lartg(hc[col], hc[col + 1], c, s, mag);
            gc[col] = c;
            gs[col] = s;
            hc[col] = mag;
            hc[col + 1] = 0.0;
            H t;
            if constexpr (S<T>::complex) t = -std::conj(s) * S_[col];
            else t = -s * S_[col];
            S_[col] = c * S_[col];
            S_[col + 1] = t;
            presid = std::abs(t);
            iters++;
            if (presid <= ptol || breakdown) break;
        }
        if (col == m) col = m - 1;
        // back substitution on the (col+1) x (col+1) upper triangle
        if (h[(size_t)col * (m + 1) + col] == H(0.0)) S_[col] = 0.0;
        for (int k = 0; k <= col; k++) y[k] = S_[k];
        for (int k = col; k > 0; k--) {
            if (y[k] != H(0.0)) {
                y[k] /= h[(size_t)k * (m + 1) + k];
                const H tk = y[k];
                for (int q = 0; q < k; q++) y[q] -= tk * h[(size_t)k * (m + 1) + q];
            }
        }
        if (y[0] != H(0.0)) y[0] /= h[0];
        for (int k = 0; k <= col; k++) hbuf[k] = S<T>::from_h(y[k]);
        FLG_CUDA(cudaMemcpyAsync(hdev, hbuf.data(), sizeof(T) * (col + 1), cudaMemcpyHostToDevice, st));
        gemv_add_kernel<T><<<grid(n), 256, 0, st>>>(V, n, col + 1, hdev, x, n);
        FLG_LAUNCH_CHECK();
        return FLG_OK;
    }

    // SciPy gmres on A x = b from the given x (x overwritten); iters += inner iterations.
    // Returns FLG_OK (converged), FLG_ERR_NOT_CONVERGED (maxiter cycles), or an error.
    // A caller that knows ||b|| (bnorm >= 0) and that x is zero (x_zero) saves the host
    // round trips that would find them out; the arithmetic is the same.
    int solve(const T *b, T *x, double rtol, int maxiter, int &iters, double &rnorm_out, double bnorm = -1.0,
              bool x_zero = false) {
        const double eps = 2.220446049250313e-16;
        double bnrm2 = bnorm;
        if (bnrm2 < 0.0) FLG_TRY(norm(b, &bnrm2));
        if (bnrm2 == 0.0) {
            FLG_CUDA(cudaMemcpyAsync(x, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
            rnorm_out = 0.0;
            return FLG_OK;
        }
        const double atol = rtol * bnrm2;
        double Mb_nrm2 = bnrm2;
        if (M) {
            FLG_TRY(M(b, tmp));
            FLG_TRY(norm(tmp, &Mb_nrm2));
        }
        double ptol_max_factor = 1.0;
        double ptol = Mb_nrm2 * std::min(ptol_max_factor, atol / bnrm2);
        double presid = 0.0, rnorm = 0.0;
        Scratch hs(m);
        bool have_r = false, r_is_b = false;
        for (int it = 0; it < maxiter; it++) {
            if (it == 0) {
                int nz = 0;
                if (!x_zero) {
                    FLG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
                    any_nonzero_kernel<<<grid(n * (S<T>::complex ? 2 : 1)), 256, 0, st>>>(
                        (const double *)x, n * (S<T>::complex ? 2 : 1), flag);
                    FLG_LAUNCH_CHECK();
                    FLG_CUDA(cudaMemcpyAsync(&nz, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
                    FLG_CUDA(cudaStreamSynchronize(st));
                }
                if (nz) {
                    FLG_TRY(residual(b, x));
                } else {
                    FLG_CUDA(cudaMemcpyAsync(r, b, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
                    r_is_b = true;
                }
                double rn0 = bnrm2;  // r == b
                if (!r_is_b) FLG_TRY(norm(r, &rn0));
                if (rn0 < atol) {
                    rnorm_out = rn0;
                    return FLG_OK;
                }
                have_r = true;
            }
            (void)have_r;
            // v0 = M^-1 r / ||M^-1 r||  (r == b on the first cycle from x = 0: M^-1 b is in tmp)
            if (it == 0 && M && r_is_b) {
                FLG_CUDA(cudaMemcpyAsync(V, tmp, sizeof(T) * n, cudaMemcpyDeviceToDevice, st));
            } else {
                FLG_TRY(precond(r, V));
            }
            double tmpn;
            FLG_TRY(norm(V, &tmpn));
            if (tmpn == 0.0) {  // r = 0 exactly: x solves the system
                rnorm = 0.0;
                break;
            }
            bool breakdown = false;
            FLG_TRY(cycle(x, tmpn, ptol, iters, presid, breakdown, hs));
            FLG_TRY(residual(b, x));
            FLG_TRY(norm(r, &rnorm));
            if (rnorm <= atol) break;
            if (breakdown) break;
            if (presid <= ptol) ptol_max_factor = std::max(eps, 0.25 * ptol_max_factor);
            else ptol_max_factor = std::min(1.0, 1.5 * ptol_max_factor);
            ptol = presid * std::min(ptol_max_factor, atol / rnorm);
        }
        rnorm_out = rnorm;
        return rnorm <= atol ? FLG_OK : FLG_ERR_NOT_CONVERGED;
    }
};

// ---- matrix-free operator of flg_gmres --------------------------------------------
struct SumOperator {
    SumLayout L;
    SumPlan P{};
    SumRun R;
    int precision;
    cudaStream_t st;
    int apply(const double *v, double *out) {
        SumRun r = R;
        r.f = v;
        r.out = out;
        return sum_run(r, L, precision, &P, st);
    }
};

static int carve_operator(Arena &ar, int kind, int64_t N, int nf, bool ck, int precision, SumOperator &op) {
    sum_layout(kind, N, N, nf, ck, precision, op.L);
    const size_t need = sum_workspace_bytes(kind, N, N, nf, ck, precision);
    char *base = ar.take<char>(need);
    if (!base) return FLG_ERR_INVALID;
    FLG_TRY(sum_plan_carve(base, need, N, N, op.L, precision, &op.P));
    op.precision = precision;
    return FLG_OK;
}

template <typename T>
static size_t gmres_bytes(int64_t N, int restart, bool ck, int precision) {
    CountingArena c;
    const int64_t n = 3 * N;
    const int nf = (sizeof(T) == 16) ? 2 : 1;
    Gmres<T>::carve_sizes(n, restart, c);
    c.take<char>(sum_workspace_bytes(0, N, N, nf, ck, FLG_PREC_FP64));
    if (precision == FLG_PREC_MIXED) {
        Gmres<T>::carve_sizes(n, restart, c);  // inner solver
        c.take<char>(sum_workspace_bytes(0, N, N, nf, ck, FLG_PREC_MIXED));
        c.take<T>(n);  // correction
    }
    return c.bytes();
}

template <typename T>
static int gmres_run(int kind, double are, double aim, const double *X, const double *eps, int64_t N, double mu_re,
                     double mu_im, const T *b, T *x, double rtol, int restart, int maxiter, int precision,
                     double inner_rtol, int *iters, int *outer, double *resid, void *work, size_t work_bytes,
                     cudaStream_t st) {
    const int64_t n = 3 * N;
    const bool ck = kind == FLG_BRINKMANLET && aim != 0.0;
    const int nf = S<T>::complex ? 2 : 1;
    Arena ar(work, work_bytes);
    Gmres<T> g;
    g.st = st;
    FLG_REQUIRE(g.carve(n, restart, ar), "workspace too small for GMRES (%zu bytes)", work_bytes);
    SumOperator op64;
    FLG_REQUIRE(carve_operator(ar, kind, N, nf, ck, FLG_PREC_FP64, op64) == FLG_OK, "workspace too small");
    op64.st = st;
    op64.R = SumRun{kind, X, N, X, eps, nullptr, N, are, aim, mu_re, mu_im, nullptr, S<T>::complex ? 1 : 0};
    g.A = [&](const T *v, T *out) { return op64.apply((const double *)v, (double *)out); };
    *iters = 0;
    *outer = 0;
    double rn = 0.0, bn = 0.0;
    if (precision == FLG_PREC_FP64) {
        int st_ = g.solve(b, x, rtol, maxiter, *iters, rn);
        if (st_ != FLG_OK && st_ != FLG_ERR_NOT_CONVERGED) return st_;
        FLG_TRY(g.norm(b, &bn));
        *resid = bn > 0 ? rn / bn : 0.0;
        if (st_ == FLG_ERR_NOT_CONVERGED) {
            set_error("GMRES did not converge (flag %d)", maxiter);
            return FLG_ERR_NOT_CONVERGED;
        }
        return FLG_OK;
    }
    // mixed: FP64 outer residual, inner GMRES on FP32-far / FP64-near matvecs
    Gmres<T> gi;
    gi.st = st;
    FLG_REQUIRE(gi.carve(n, restart, ar), "workspace too small for GMRES");
    SumOperator opm;
    FLG_REQUIRE(carve_operator(ar, kind, N, nf, ck, FLG_PREC_MIXED, opm) == FLG_OK, "workspace too small");
    opm.st = st;
    opm.R = op64.R;
    T *d = ar.take<T>(n);
    FLG_REQUIRE(d != nullptr, "workspace too small");
    FLG_TRY(sum_plan_geometry(X, eps, N, opm.L, &opm.P, st));
    gi.A = [&](const T *v, T *out) { return opm.apply((const double *)v, (double *)out); };
    FLG_TRY(g.norm(b, &bn));
    if (bn == 0.0) {
        FLG_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * n, st));
        *resid = 0.0;
        return FLG_OK;
    }
    const int max_outer = 40;
    double prev = INFINITY;
    int stall = 0;
    for (int o = 0; o <= max_outer; o++) {
        bool is_b = false;
        FLG_TRY(o == 0 ? g.residual_from(b, x, &is_b) : g.residual(b, x));
        if (is_b) rn = bn;
        else FLG_TRY(g.norm(g.r, &rn));
        *resid = rn / bn;
        if (rn <= rtol * bn) return FLG_OK;
        if (o == max_outer || *iters >= restart * maxiter) break;
        stall = (rn > 0.5 * prev) ? stall + 1 : 0;
        if (stall >= 3) break;
        prev = rn;
        FLG_CUDA(cudaMemsetAsync(d, 0, sizeof(T) * n, st));
        double rin = 0.0;
        int s2 = gi.solve(g.r, d, inner_rtol, std::max(1, maxiter), *iters, rin, rn, true);
        if (s2 != FLG_OK && s2 != FLG_ERR_NOT_CONVERGED) return s2;
        add_kernel<T><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(x, d, n);
        FLG_LAUNCH_CHECK();
        (*outer)++;
    }
    set_error("GMRES iterative refinement did not converge: residual %.3e after %d refinement steps", *resid,
              *outer);
    return FLG_ERR_NOT_CONVERGED;
}

// ---- dense GMRES-IR (flg_gmres_ir_dense) -------------------------------------------
int gemv_f32_presplit(int64_t n_rows, int64_t n_cols, const float *A, int64_t ld, const double *x, float *xsplit,
                      double *y, cudaStream_t st);
int lu_solve_lowp_apply(int64_t n, const float *LU, int64_t ld, const float *dinv, const double *b, double *x,
                        void *work, size_t work_bytes, cudaStream_t st);
size_t lu_solve_lowp_bytes(int64_t n);

}  // namespace flg

using namespace flg;

extern "C" size_t flg_gmres_workspace(int64_t N, int restart, int is_complex, int precision) {
    if (N < 0 || restart < 1) return 0;
    const bool ck = true;  // size for the larger (complex-kernel) accumulator layout
    return is_complex ? gmres_bytes<double2>(N, restart, ck, precision)
                      : gmres_bytes<double>(N, restart, false, precision);
}

extern "C" int flg_gmres(int kind, double alpha_re, double alpha_im, const double *X, const double *eps, int64_t N,
                         double mu_re, double mu_im, const double *b, double *x, int is_complex, double rtol,
                         int restart, int maxiter, int precision, double inner_rtol, int *iters, int *outer,
                         double *resid, void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_gmres");
    FLG_TRY(check_kernel_args(kind, alpha_re, alpha_im));
    FLG_REQUIRE(N >= 0 && restart >= 1 && maxiter >= 1, "bad GMRES sizes");
    FLG_REQUIRE(rtol >= 0.0 && inner_rtol > 0.0, "tolerances must be non-negative");
    FLG_REQUIRE(precision == FLG_PREC_FP64 || precision == FLG_PREC_MIXED, "unknown precision");
    FLG_REQUIRE(iters && outer && resid, "null output pointer");
    const bool cplx_needed = (kind == FLG_BRINKMANLET && alpha_im != 0.0) || mu_im != 0.0;
    FLG_REQUIRE(is_complex || !cplx_needed, "a complex kernel or viscosity needs complex vectors");
    FLG_REQUIRE(!(mu_re == 0.0 && mu_im == 0.0), "mu must be non-zero");
    *iters = 0;
    *outer = 0;
    *resid = 0.0;
    if (N == 0) return FLG_OK;
    restart = (int)std::min<int64_t>(restart, 3 * N);
    cudaStream_t st = as_stream(stream);
    if (is_complex)
        return gmres_run<double2>(kind, alpha_re, alpha_im, X, eps, N, mu_re, mu_im, (const double2 *)b, (double2 *)x,
                                  rtol, restart, maxiter, precision, inner_rtol, iters, outer, resid, work,
                                  work_bytes, st);
    return gmres_run<double>(kind, alpha_re, alpha_im, X, eps, N, mu_re, mu_im, b, x, rtol, restart, maxiter,
                             precision, inner_rtol, iters, outer, resid, work, work_bytes, st);
}

extern "C" size_t flg_gmres_ir_dense_workspace(int64_t n, int restart) {
    if (n < 0 || restart < 1) return 0;
    CountingArena c;
    Gmres<double>::carve_sizes(n, restart, c);  // outer residual
    Gmres<double>::carve_sizes(n, restart, c);  // inner preconditioned solve
    c.take<double>(n);                          // correction
    c.take<char>(lu_solve_lowp_bytes(n));
    c.take<float>(2 * n);                       // x split into FP32 parts for the inner matvec
    return c.bytes();
}

extern "C" int flg_gmres_ir_dense(int64_t n, const double *A, int64_t ld, const float *A32, int64_t lda32,
                                  const float *LU32, int64_t ld32, const float *dinv, const double *b, double *x, double rtol, int restart, int maxiter, int *iters,
                                  int *outer, double *resid, void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_gmres_ir_dense");
    FLG_REQUIRE(n >= 0 && ld >= n && ld32 >= n && restart >= 1 && maxiter >= 1, "bad GMRES-IR arguments");
    FLG_REQUIRE(iters && outer && resid, "null output pointer");
    *iters = 0;
    *outer = 0;
    *resid = 0.0;
    if (n == 0) return FLG_OK;
    restart = (int)std::min<int64_t>(restart, n);
    cudaStream_t st = as_stream(stream);
    Arena ar(work, work_bytes);
    Gmres<double> g, gi;
    g.st = gi.st = st;
    FLG_REQUIRE(g.carve(n, restart, ar) && gi.carve(n, restart, ar), "workspace too small for GMRES-IR");
    double *d = ar.take<double>(n);
    const size_t lsb = lu_solve_lowp_bytes(n);
    char *lw = ar.take<char>(lsb);
    float *xs = ar.take<float>(2 * n);
    FLG_REQUIRE(d && lw && xs, "workspace too small for GMRES-IR");
    // outer residuals with the FP64 matrix; inner (preconditioned, tolerance 1e-4) matvecs
    // with the FP32 copy when the caller provides one
    g.A = [&](const double *v, double *out) { return flg_gemv_f64(n, n, A, ld, v, out, st); };
    if (A32)
        gi.A = [&](const double *v, double *out) { return gemv_f32_presplit(n, n, A32, lda32, v, xs, out, st); };
    else
        gi.A = g.A;
    gi.M = [&](const double *v, double *out) { return lu_solve_lowp_apply(n, LU32, ld32, dinv, v, out, lw, lsb, st); };
    double bn;
    FLG_TRY(g.norm(b, &bn));
    if (bn == 0.0) {
        FLG_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
        return FLG_OK;
    }
    const double inner = 1e-4;
    double rn = 0.0, prev = INFINITY;
    int stall = 0;
    for (int o = 0; o <= 60; o++) {
        bool is_b = false;
        FLG_TRY(o == 0 ? g.residual_from(b, x, &is_b) : g.residual(b, x));
        if (is_b) rn = bn;
        else FLG_TRY(g.norm(g.r, &rn));
        *resid = rn / bn;
        if (rn <= rtol * bn) return FLG_OK;
        if (*iters >= restart * maxiter) break;
        stall = (rn > 0.5 * prev) ? stall + 1 : 0;
        if (stall >= 3) break;
        prev = rn;
        FLG_CUDA(cudaMemsetAsync(d, 0, sizeof(double) * n, st));
        double rin;
        int s2 = gi.solve(g.r, d, inner, maxiter, *iters, rin, rn, true);
        if (s2 != FLG_OK && s2 != FLG_ERR_NOT_CONVERGED) return s2;
        add_kernel<double><<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(x, d, n);
        FLG_LAUNCH_CHECK();
        (*outer)++;
    }
    set_error("GMRES-IR did not converge: residual %.3e after %d refinement steps", *resid, *outer);
    return FLG_ERR_NOT_CONVERGED;
}
