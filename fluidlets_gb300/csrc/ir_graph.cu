// ir_graph.cu -- FP64 GMRES-based iterative refinement as one CUDA graph.
//
// flg_gmres_ir_dense (krylov.cu) drives the refinement from the host and reads
// the Hessenberg column back after every Arnoldi step.  Here the same algorithm
// runs without the host: every scalar (norms, the Hessenberg matrix, the Givens
// rotations, the least-squares right-hand side, the tolerances, the counters)
// lives in a device state block updated by single-thread control kernels, and
// the two loops are conditional WHILE nodes of a CUDA graph whose conditions the
// control kernels set with cudaGraphSetConditional:
//
//   x = 0, r = b, ||b||                              (prologue)
//   WHILE the residual is above rtol ||b||:          (refinement steps)
//     v0 = M^-1 r, beta = ||v0||, ptol = 1e-4 beta   (inner GMRES on M^-1 A d = M^-1 r)
//     WHILE the inner residual estimate is above ptol and columns remain:
//       w = M^-1 (A32 v_k); two classical Gram-Schmidt passes; Givens update
//     x += V y (upper-triangular least squares)
//     r = b - K x (FP64), ||r||, stall and step-count checks
//
// M^-1 is the low-precision LU's dataflow solve (lu.cu), A32 the FP32 copy of K
// multiplied with a compensated FP32 product, K the FP64 matrix.  The arithmetic
// follows flg_gmres_ir_dense step for step (SciPy's GMRES semantics for the inner
// solve: zero start, known ||r||, one restart cycle of at most m columns; CGS2;
// LAPACK lartg rotations).  The multi-vector kernels read the current column count
// from the state block, so one captured body serves every iteration.  A replay
// costs no host round trip: the host reads the state once, at the end.
#include <algorithm>
#include <cmath>

#include "flg_common.cuh"

namespace flg {

int gemv_f32_presplit(int64_t n_rows, int64_t n_cols, const float *A, int64_t ld, const double *x, float *xsplit,
                      double *y, cudaStream_t st);
int lu_solve_lowp_apply(int64_t n, const float *LU, int64_t ld, const float *dinv, const double *b, double *x,
                        void *work, size_t work_bytes, cudaStream_t st);
size_t lu_solve_lowp_bytes(int64_t n);
int lu_solve_lowp_prepare();

constexpr int kIrMaxM = 64;             // inner columns at most
constexpr int kIrThreads = 256;
constexpr int64_t kIrChunk = 8192;      // elements per CTA of a dot product
constexpr double kIrInner = 1e-4;       // inner (preconditioned) tolerance
constexpr double kEps = 2.220446049250313e-16;

// the device state of one refinement (one graph)
struct IrState {
    double bn, tol, rn, prev_rn;
    double beta, ptol, presid;
    double h[kIrMaxM * (kIrMaxM + 1)];  // column-major: column c at h + c (m + 1)
    double g[kIrMaxM + 1];              // the rotated right-hand side
    double cs[kIrMaxM], sn[kIrMaxM];
    double y[kIrMaxM];
    double d1[kIrMaxM + 1], d2[kIrMaxM + 1];  // the two Gram-Schmidt passes' coefficients
    double nb, na;                      // |w|^2 before and after the passes
    double hnext;                       // |w| after the passes: the new column's divisor
    double dot;                         // a single dot product's result (b.b, v0.v0, r.r)
    int m;                              // inner columns allowed
    int k;                              // inner columns done in this step
    int breakdown;
    int outer, max_outer, iters, stall;
    int status;                         // 0 running, 1 converged, 2 stopped (stall / step limit)
};

// partial[v * nchunk + c] = sum over chunk c of V[v] . w, for v < nvec (nvec from the state
// when count_k, else 1); CTAs beyond the current count return at once
__global__ void __launch_bounds__(kIrThreads) ir_dot_partial(const double *V, int64_t n, const double *w,
                                                             int64_t nchunk, double *partial, const IrState *S,
                                                             bool count_k) {
    const int v = blockIdx.y;
    const int nvec = count_k ? S->k + 1 : 1;
    if (v >= nvec) return;
    __shared__ double sm[kIrThreads / 32];
    const double *a = V + (int64_t)v * n;
    const int64_t c = blockIdx.x, lo = c * kIrChunk, hi = min(n, lo + kIrChunk);
    double acc = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += kIrThreads) acc = fma(a[i], w[i], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < kIrThreads / 32; q++) s += sm[q];
        partial[(int64_t)v * nchunk + c] = s;
    }
}

// out[v] = in-order sum of the partials (deterministic)
__global__ void ir_dot_finish(const double *partial, int64_t nchunk, double *out, const IrState *S, bool count_k) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const int nvec = count_k ? S->k + 1 : 1;
    if (v >= nvec) return;
    double s = 0.0;
    for (int64_t c = 0; c < nchunk; c++) s += partial[(int64_t)v * nchunk + c];
    out[v] = s;
}

// w -= sum_{v <= k} V[v] coef[v]
__global__ void ir_sub(const double *V, int64_t n, const double *coef, double *w, const IrState *S) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nvec = S->k + 1;
    double acc = w[i];
    for (int v = 0; v < nvec; v++) acc -= V[(int64_t)v * n + i] * coef[v];
    w[i] = acc;
}

// dst = V[k] (the current column, into a fixed buffer for the matrix-vector product)
__global__ void ir_copy_col(const double *V, int64_t n, double *dst, const IrState *S) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = V[(int64_t)S->k * n + i];
}

// V[k] = w / h(k, k - 1) after a step (k already advanced), unless the step broke down
__global__ void ir_store_col(const double *w, int64_t n, double *V, const IrState *S) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || S->breakdown) return;
    V[(int64_t)S->k * n + i] = w[i] * (1.0 / S->hnext);
}

// V[0] *= 1 / beta
__global__ void ir_scale0(double *V, int64_t n, const IrState *S) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && S->beta > 0.0) V[i] *= 1.0 / S->beta;
}

// x += sum_{v < k} V[v] y[v]
__global__ void ir_update_x(const double *V, int64_t n, double *x, const IrState *S) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nvec = S->k;
    double acc = 0.0;
    for (int v = 0; v < nvec; v++) acc += V[(int64_t)v * n + i] * S->y[v];
    x[i] += acc;
}

// r = b - y (y = K x on entry, in r)
__global__ void ir_rsub(const double *b, double *r, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = b[i] - r[i];
}

// ---- control (one thread) -------------------------------------------------------
// prologue: ||b||, the refinement's tolerance, r = b (x = 0)
__global__ void ir_ctrl_init(IrState *S, double rtol, int m, int max_outer, cudaGraphConditionalHandle h_outer) {
    S->bn = sqrt(fmax(S->dot, 0.0));
    S->tol = rtol * S->bn;
    S->rn = S->bn;
    S->prev_rn = INFINITY;
    S->m = m;
    S->k = 0;
    S->outer = 0;
    S->max_outer = max_outer;
    S->iters = 0;
    S->stall = 0;
    S->status = S->rn <= S->tol ? 1 : 0;  // b = 0: x = 0 is the answer
    cudaGraphSetConditional(h_outer, S->status == 0 ? 1u : 0u);
}

// start of an inner solve: beta = ||M^-1 r||, its tolerance, g = beta e1
__global__ void ir_ctrl_inner_init(IrState *S, cudaGraphConditionalHandle h_inner) {
    S->beta = sqrt(fmax(S->dot, 0.0));
    S->ptol = S->beta * kIrInner;
    for (int q = 0; q <= S->m; q++) S->g[q] = 0.0;
    S->g[0] = S->beta;
    S->k = 0;
    S->breakdown = 0;
    cudaGraphSetConditional(h_inner, S->beta > 0.0 ? 1u : 0u);
}

// LAPACK lartg for real arguments: c f + s g = r, -s f + c g = 0
__device__ void ir_lartg(double f, double g, double &c, double &s, double &r) {
    if (g == 0.0) {
        c = 1.0;
        s = 0.0;
        r = f;
    } else if (f == 0.0) {
        c = 0.0;
        s = g > 0 ? 1.0 : -1.0;
        r = fabs(g);
    } else {
        const double d = hypot(f, g);
        c = fabs(f) / d;
        r = f > 0 ? d : -d;
        s = g / r;
    }
}

// after an Arnoldi step: the new Hessenberg column, the previous rotations applied, a new one
// made, the residual estimate; the inner loop goes on while it exceeds ptol and columns remain
__global__ void ir_ctrl_step(IrState *S, cudaGraphConditionalHandle h_inner) {
    const int col = S->k, m = S->m;
    double *hc = S->h + col * (m + 1);
    for (int q = 0; q <= col; q++) hc[q] = S->d1[q] + S->d2[q];
    const double h0 = sqrt(fmax(S->nb, 0.0)), h1n = sqrt(fmax(S->na, 0.0));
    hc[col + 1] = h1n;
    S->hnext = h1n;
    if (h1n <= kEps * h0) {
        hc[col + 1] = 0.0;
        S->breakdown = 1;
    }
    for (int q = 0; q < col; q++) {
        const double c = S->cs[q], sn = S->sn[q], n0 = hc[q], n1 = hc[q + 1];
        hc[q] = c * n0 + sn * n1;
        hc[q + 1] = -sn * n0 + c * n1;
    }
    double c, sn, mag;
    ir_lartg(hc[col], hc[col + 1], c, sn, mag);
    S->cs[col] = c;
    S->sn[col] = sn;
    hc[col] = mag;
    hc[col + 1] = 0.0;
    const double t = -sn * S->g[col];
    S->g[col] = c * S->g[col];
    S->g[col + 1] = t;
    S->presid = fabs(t);
    S->iters++;
    S->k = col + 1;
    const bool more = S->presid > S->ptol && !S->breakdown && S->k < m;
    cudaGraphSetConditional(h_inner, more ? 1u : 0u);
}

// the least-squares solution y of the k x k upper-triangular system
__global__ void ir_ctrl_back(IrState *S) {
    const int kk = S->k, m = S->m;
    if (kk == 0) return;
    const int col = kk - 1;
    double *h = S->h, *y = S->y;
    if (h[col * (m + 1) + col] == 0.0) S->g[col] = 0.0;
    for (int q = 0; q <= col; q++) y[q] = S->g[q];
    for (int c = col; c > 0; c--) {
        if (y[c] != 0.0) {
            y[c] /= h[c * (m + 1) + c];
            const double tk = y[c];
            for (int q = 0; q < c; q++) y[q] -= tk * h[c * (m + 1) + q];
        }
    }
    if (y[0] != 0.0) y[0] /= h[0];
}

// after a refinement step: ||r||, convergence, stagnation and the step limit
__global__ void ir_ctrl_outer(IrState *S, cudaGraphConditionalHandle h_outer) {
    S->rn = sqrt(fmax(S->dot, 0.0));
    S->outer++;
    int go = 1;
    if (S->rn <= S->tol) {
        S->status = 1;
        go = 0;
    } else {
        S->stall = S->rn > 0.5 * S->prev_rn ? S->stall + 1 : 0;
        S->prev_rn = S->rn;
        if (S->stall >= 3 || S->outer >= S->max_outer) {
            S->status = 2;
            go = 0;
        }
    }
    cudaGraphSetConditional(h_outer, (unsigned)go);
}

}  // namespace flg

using namespace flg;

namespace {

struct IrLayout {
    IrState *S = nullptr;
    double *r = nullptr, *V = nullptr, *w = nullptr, *vk = nullptr, *tmp = nullptr, *partial = nullptr;
    float *xs = nullptr;
    char *aw = nullptr;
    size_t awb = 0;
    int64_t nchunk = 0;
};

template <class Ar>
void ir_carve(Ar &ar, int64_t n, int m, IrLayout &L) {
    L.nchunk = ceil_div(std::max<int64_t>(n, 1), kIrChunk);
    L.S = ar.template take<IrState>(1);
    L.r = ar.template take<double>(n);
    L.V = ar.template take<double>((size_t)(m + 1) * n);
    L.w = ar.template take<double>(n);
    L.vk = ar.template take<double>(n);
    L.tmp = ar.template take<double>(n);
    L.partial = ar.template take<double>((size_t)(m + 1) * L.nchunk);
    L.xs = ar.template take<float>(2 * n);
    L.awb = lu_solve_lowp_bytes(n);
    L.aw = ar.template take<char>(L.awb);
}

// out = V[0..count) . w (count = k + 1 from the state when multi, else 1) on stream s
int ir_dots(const IrLayout &L, int64_t n, int m, const double *V, const double *w, double *out, bool multi,
            cudaStream_t s) {
    ir_dot_partial<<<dim3((unsigned)L.nchunk, multi ? (unsigned)(m + 1) : 1u), kIrThreads, 0, s>>>(V, n, w, L.nchunk,
                                                                                             L.partial, L.S, multi);
    FLG_LAUNCH_CHECK();
    ir_dot_finish<<<(unsigned)ceil_div(m + 1, 64), 64, 0, s>>>(L.partial, L.nchunk, out, L.S, multi);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

}  // namespace

extern "C" size_t flg_gmres_ir_graph_workspace(int64_t n, int m) {
    if (n < 0 || m < 1 || m > kIrMaxM) return 0;
    CountingArena c;
    IrLayout L;
    ir_carve(c, n, m, L);
    return c.bytes();
}

// The refinement of K x = b as an instantiated graph over fixed buffers (see the file comment).
extern "C" int flg_gmres_ir_graph_create(int64_t n, const double *K, int64_t ld, const float *A32, int64_t lda32,
                                         const float *LU32, int64_t ld32, const float *dinv, const double *b,
                                         double *x, double rtol, int m, int max_outer, void *work,
                                         size_t work_bytes, void *stream, void **graph_exec) {
    FLG_RANGE("flg_gmres_ir_graph_create");
    FLG_REQUIRE(graph_exec, "null graph handle");
    *graph_exec = nullptr;
    FLG_REQUIRE(n >= 1 && ld >= n && lda32 >= n && ld32 >= n, "bad GMRES-IR graph sizes");
    FLG_REQUIRE(m >= 1 && m <= kIrMaxM, "inner columns must lie in [1, %d]", kIrMaxM);
    FLG_REQUIRE(max_outer >= 1 && rtol >= 0.0, "bad GMRES-IR graph limits");
    FLG_REQUIRE(K && A32 && LU32 && dinv && b && x, "null pointer");
    FLG_REQUIRE(stream, "graph capture needs a non-default stream");
    m = (int)std::min<int64_t>(m, n);
    Arena ar(work, work_bytes);
    IrLayout L;
    ir_carve(ar, n, m, L);
    FLG_REQUIRE(L.aw != nullptr, "workspace too small for the GMRES-IR graph (%zu bytes)", work_bytes);
    FLG_TRY(lu_solve_lowp_prepare());
    cudaStream_t st = as_stream(stream), s2 = nullptr, s3 = nullptr;
    FLG_CUDA(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking));
    FLG_CUDA(cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking));
    ProfSuppress quiet;
    const unsigned gridn = (unsigned)ceil_div(n, 256);
    IrState *S = L.S;
    cudaGraph_t g = nullptr, body_out = nullptr, body_in = nullptr;
    cudaGraphConditionalHandle h_outer = 0, h_inner = 0;
    int rc = FLG_OK;
    auto body = [&]() -> int {
        // prologue on st: x = 0, r = b, ||b||, the tolerance, the outer condition
        FLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        FLG_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));
        FLG_CUDA(cudaMemcpyAsync(L.r, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        FLG_TRY(ir_dots(L, n, m, b, b, &S->dot, false, st));
        // the outer loop's handle belongs to the graph being captured on st
        cudaStreamCaptureStatus cs;
        FLG_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
        FLG_CUDA(cudaGraphConditionalHandleCreate(&h_outer, g, 0, 0));
        ir_ctrl_init<<<1, 1, 0, st>>>(S, rtol, m, max_outer, h_outer);
        FLG_LAUNCH_CHECK();
        {
            const cudaGraphNode_t *deps = nullptr;
            size_t ndeps = 0;
            FLG_CUDA(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &ndeps));
            cudaGraphNodeParams p = {};
            p.type = cudaGraphNodeTypeConditional;
            p.conditional.handle = h_outer;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t node;
            FLG_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p));
            FLG_CUDA(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            body_out = p.conditional.phGraph_out[0];
        }
        // one refinement step, captured on s2 into the outer loop's body
        FLG_CUDA(cudaStreamBeginCaptureToGraph(s2, body_out, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        FLG_TRY(lu_solve_lowp_apply(n, LU32, ld32, dinv, L.r, L.V, L.aw, L.awb, s2));  // v0 = M^-1 r
        FLG_TRY(ir_dots(L, n, m, L.V, L.V, &S->dot, false, s2));
        FLG_CUDA(cudaGraphConditionalHandleCreate(&h_inner, body_out, 0, 0));
        ir_ctrl_inner_init<<<1, 1, 0, s2>>>(S, h_inner);
        FLG_LAUNCH_CHECK();
        ir_scale0<<<gridn, 256, 0, s2>>>(L.V, n, S);
        FLG_LAUNCH_CHECK();
        {
            cudaStreamCaptureStatus cs2;
            const cudaGraphNode_t *deps = nullptr;
            size_t ndeps = 0;
            FLG_CUDA(cudaStreamGetCaptureInfo(s2, &cs2, nullptr, nullptr, &deps, nullptr, &ndeps));
            cudaGraphNodeParams p = {};
            p.type = cudaGraphNodeTypeConditional;
            p.conditional.handle = h_inner;
            p.conditional.type = cudaGraphCondTypeWhile;
            p.conditional.size = 1;
            cudaGraphNode_t node;
            FLG_CUDA(cudaGraphAddNode(&node, body_out, deps, nullptr, ndeps, &p));
            FLG_CUDA(cudaStreamUpdateCaptureDependencies(s2, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
            body_in = p.conditional.phGraph_out[0];
        }
        // one Arnoldi step, captured on s3 into the inner loop's body
        FLG_CUDA(cudaStreamBeginCaptureToGraph(s3, body_in, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        ir_copy_col<<<gridn, 256, 0, s3>>>(L.V, n, L.vk, S);
        FLG_LAUNCH_CHECK();
        FLG_TRY(gemv_f32_presplit(n, n, A32, lda32, L.vk, L.xs, L.tmp, s3));
        FLG_TRY(lu_solve_lowp_apply(n, LU32, ld32, dinv, L.tmp, L.w, L.aw, L.awb, s3));
        FLG_TRY(ir_dots(L, n, m, L.w, L.w, &S->nb, false, s3));
        FLG_TRY(ir_dots(L, n, m, L.V, L.w, S->d1, true, s3));
        ir_sub<<<gridn, 256, 0, s3>>>(L.V, n, S->d1, L.w, S);
        FLG_LAUNCH_CHECK();
        FLG_TRY(ir_dots(L, n, m, L.V, L.w, S->d2, true, s3));
        ir_sub<<<gridn, 256, 0, s3>>>(L.V, n, S->d2, L.w, S);
        FLG_LAUNCH_CHECK();
        FLG_TRY(ir_dots(L, n, m, L.w, L.w, &S->na, false, s3));
        ir_ctrl_step<<<1, 1, 0, s3>>>(S, h_inner);
        FLG_LAUNCH_CHECK();
        ir_store_col<<<gridn, 256, 0, s3>>>(L.w, n, L.V, S);
        FLG_LAUNCH_CHECK();
        cudaGraph_t got = nullptr;
        FLG_CUDA(cudaStreamEndCapture(s3, &got));
        // the rest of the step on s2: x += V y, r = b - K x, ||r||, the outer condition
        ir_ctrl_back<<<1, 1, 0, s2>>>(S);
        FLG_LAUNCH_CHECK();
        ir_update_x<<<gridn, 256, 0, s2>>>(L.V, n, x, S);
        FLG_LAUNCH_CHECK();
        FLG_TRY(flg_gemv_f64(n, n, K, ld, x, L.r, s2));
        ir_rsub<<<gridn, 256, 0, s2>>>(b, L.r, n);
        FLG_LAUNCH_CHECK();
        FLG_TRY(ir_dots(L, n, m, L.r, L.r, &S->dot, false, s2));
        ir_ctrl_outer<<<1, 1, 0, s2>>>(S, h_outer);
        FLG_LAUNCH_CHECK();
        FLG_CUDA(cudaStreamEndCapture(s2, &got));
        FLG_CUDA(cudaStreamEndCapture(st, &g));
        return FLG_OK;
    };
    rc = body();
    if (rc != FLG_OK) {  // end any capture still open, keep the first error's text
        cudaGraph_t junk = nullptr;
        for (cudaStream_t s : {s3, s2, st}) {
            cudaStreamCaptureStatus cs;
            if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                cudaStreamEndCapture(s, &junk);
                if (junk && s == st) cudaGraphDestroy(junk);
                junk = nullptr;
            }
        }
        cudaGetLastError();
        g = nullptr;
    }
    cudaStreamDestroy(s2);
    cudaStreamDestroy(s3);
    if (rc != FLG_OK) return rc;
    cudaGraphExec_t ge = nullptr;
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_error("GMRES-IR graph instantiation failed: %s", cudaGetErrorString(e));
        return FLG_ERR_CUDA;
    }
    *graph_exec = (void *)ge;
    return FLG_OK;
}

// The outcome of the last replay (synchronizes `stream`): inner iterations, refinement steps,
// the final ||b - K x|| / ||b|| with the FP64 K; FLG_OK if it met rtol, FLG_ERR_NOT_CONVERGED
// if it stopped on stagnation or the step limit.
extern "C" int flg_gmres_ir_graph_result(const void *work, int *iters, int *outer, double *resid, void *stream) {
    FLG_REQUIRE(work && iters && outer && resid, "null pointer");
    IrState h;
    cudaStream_t st = as_stream(stream);
    Arena ar(const_cast<void *>(work), sizeof(IrState) + 512);  // the state is the first slice
    const IrState *S = ar.take<IrState>(1);
    FLG_CUDA(cudaMemcpyAsync(&h, S, sizeof(IrState), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    *iters = h.iters;
    *outer = h.outer;
    *resid = h.bn > 0.0 ? h.rn / h.bn : 0.0;
    if (h.status == 1) return FLG_OK;
    set_error("GMRES-IR did not converge: residual %.3e after %d refinement steps", *resid, h.outer);
    return FLG_ERR_NOT_CONVERGED;
}
