// lu.cu -- dense LU factorizations and triangular solves.
//
// FP64 (the drop-in for scipy.linalg.solve, core/solve.py:64-67, and
// np.linalg.solve, swimming.py:101): right-looking blocked LU with partial
// pivoting, row-major storage, block width kPanel = 64.
//   panel_f64_kernel  cooperative launch over up to one CTA per SM; each CTA
//                     keeps a slab of panel rows in shared memory; one round of
//                     published candidates per column (pivot search is a
//                     grid-wide argmax, first index on ties as LAPACK's idamax),
//                     with the next column's look-ahead overlapping it.
//   laswp_kernel      the panel's row swaps on the other columns.
//   trsm_f64_kernel   U12 = L11^-1 A12.
//   dgemm_update      A22 -= L21 U12 (FP64 CUDA cores).
//
// Low precision (preconditioner of FP64 GMRES-IR): blocked LU WITHOUT
// pivoting in FP32 storage, block FLG_LU_LOWP_BLOCK = 128; the diagonal block
// is factored by one CTA, which also writes the inverses of its L and U
// factors (kept in `dinv` for the solves); the panels are GEMMs with those
// inverses; the trailing update runs on the tensor cores (tc_gemm.cu, deferred
// to one rank-512 update per outer panel of four blocks) or on CUDA cores
// (FLG_LU_FP32).  With the tensor cores the next diagonal block runs ahead on
// a side stream while the rest of each update finishes.
//
// Every spin-wait (the grid barrier, the solves' dataflow, waits.cuh; the
// diagonal block's warp handshake, an iteration count) is bounded and reports
// failure through a device flag instead of hanging.
#include <cooperative_groups.h>
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "flg_common.cuh"
#include "waits.cuh"

namespace flg {

constexpr int kPanel = 64;                    // FP64 LU block width
constexpr int kNB = FLG_LU_LOWP_BLOCK;        // low-precision LU block

// ---- FP64 panel ------------------------------------------------------------------
// Partial-pivoting LU of the m x kb panel A[k0:n, k0:k0+kb] (LAPACK getf2's pivot
// choice: the largest |a| in the column, the first row on ties), one cooperative
// launch of up to one CTA per SM, each CTA holding `rpc` consecutive panel rows in
// shared memory (CTA c owns rows k0 + c rpc ...).  GB300 runs FP64 at ~2 FMA per
// SM and clock, so the panel's arithmetic must be spread over every SM; what
// limits it is the exchange between CTAs per column, which is kept to one
// round of published values:
//   * every CTA publishes, for column j, its candidate (the largest |a| among its
//     rows >= g, encoded with the column's parity bit in one 64-bit word released
//     after the candidate's full row and, by the owner of row g, row g itself);
//   * every CTA polls the words (acquire), picks the winner (largest value; on ties
//     the smaller CTA index, which owns the smaller rows), and reads the winning
//     row; the winner writes ipiv[g] and row g's old content into the pivot row,
//     the owner of g writes the pivot row into row g;
//   * look-ahead inside the panel: after scaling column j each CTA updates column
//     j + 1 first, finds its next candidate, completes the update of that row and
//     of row g + 1 and publishes them, and only then updates its other rows, so
//     the bulk of the rank-1 update overlaps the exchange.
// Every element receives the same fma, in the same column order, as in the
// textbook right-looking loop, so the factors do not depend on the CTA count.
// A word holds (bits(|a|) + 1) | parity << 63 (0 for "no rows >= g" or only
// NaN); the
// parity ((j >> 1) & 1) tells column j from column j - 2, which used the same
// one of the two buffers; the host presets both buffers to parity 1 before
// every panel.
struct PanelArgs {
    double *A;
    int64_t ld, n, k0;
    int kb, rpc;
    int32_t *ipiv;
    GridBar *bar;                 // err: a wait ran out; info: 1 + first zero pivot
    unsigned long long *word;     // [2][nblk]
    double *rowbuf;               // [2][nblk][kRowBufLd]: each CTA's candidate row and 1 / its pivot
    double *diagbuf;              // [2][kb]: row g
};

__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

constexpr int kRowBufLd = kPanel + 8;  // a published row: kb values, then the reciprocal of its pivot

__global__ void __launch_bounds__(256) panel_f64_kernel(PanelArgs a) {
    extern __shared__ double P[];  // [rpc][kb]
    __shared__ double s_piv[kRowBufLd], s_old[kPanel];
    __shared__ unsigned long long red_w[8];
    __shared__ int red_c[8];
    __shared__ double s_rcp;  // 1 / this CTA's candidate value, published with its row
    __shared__ int s_win;     // winning CTA
    __shared__ int s_abort;
    const int nblk = gridDim.x, c = blockIdx.x, kb = a.kb, rpc = a.rpc;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int64_t r0 = a.k0 + (int64_t)c * rpc;
    const int nr = (int)max((int64_t)0, min((int64_t)rpc, a.n - r0));
    for (int e = t; e < nr * kb; e += blockDim.x) {
        const int lr = e / kb, j = e - lr * kb;
        P[e] = a.A[(r0 + lr) * a.ld + a.k0 + j];
    }
    if (t == 0) s_abort = 0;
    __syncthreads();

    // Local argmax of |P[., col]| over local rows >= lo (first row on ties), compared as
    // integers (the bits of a non-negative double order like its value; NaN never wins, as
    // in an FP comparison): the key bits(|a|) + 1 (0 if there is no candidate) and the local
    // row (-1), the same in every thread.  With `upd`, each row's column col first receives
    // its update from column col - 1 (multiplier P[., col - 1], pivot-row entry u).
    auto argmax = [&](int col, int lo, bool upd, double u, int &row) -> unsigned long long {
        unsigned long long best = 0;
        int brow = INT_MAX;
        for (int lr = lo + t; lr < nr; lr += blockDim.x) {
            double x = P[lr * kb + col];
            if (upd) {
                x = fma(-P[lr * kb + col - 1], u, x);
                P[lr * kb + col] = x;
            }
            const unsigned long long b = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
            const unsigned long long k = b > 0x7ff0000000000000ull ? 0ull : b + 1ull;
            if (k > best) {
                best = k;
                brow = lr;
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long ov = __shfl_xor_sync(0xffffffffu, best, o);
            const int orow = __shfl_xor_sync(0xffffffffu, brow, o);
            if (ov > best || (ov == best && orow < brow)) {
                best = ov;
                brow = orow;
            }
        }
        if (lane == 0) {
            red_w[warp] = best;
            red_c[warp] = brow;
        }
        __syncthreads();
        unsigned long long bk = red_w[0];
        int br = red_c[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); w++)
            if (red_w[w] > bk || (red_w[w] == bk && red_c[w] < br)) {
                bk = red_w[w];
                br = red_c[w];
            }
        __syncthreads();
        row = bk == 0 ? -1 : br;
        return bk;
    };
    // the reciprocal of the candidate's value, computed while other threads work (one thread)
    auto candidate_rcp = [&](int col, int cand) {
        if (t == blockDim.x - 1) {
            const double v = cand >= 0 ? P[cand * kb + col] : 0.0;
            s_rcp = (v != 0.0 && isfinite(v)) ? 1.0 / v : 0.0;
        }
    };
    // publish column col's candidate (key k, local row cand, its reciprocal s_rcp) and, from
    // the owner, row g
    auto publish = [&](int col, unsigned long long k, int cand) {
        const int buf = col & 1;
        const unsigned long long par = (unsigned long long)((col >> 1) & 1) << 63;
        const int64_t g = a.k0 + col;
        double *rb = a.rowbuf + ((int64_t)buf * nblk + c) * kRowBufLd;
        if (cand >= 0 && t < kb) rb[t] = P[cand * kb + t];
        if (cand >= 0 && t == kb) rb[kPanel] = s_rcp;
        if (g >= r0 && g < r0 + nr && t < kb) a.diagbuf[buf * kb + t] = P[(g - r0) * kb + t];
        __syncthreads();  // the CTA's writes precede thread 0's release (cumulative through bar.sync)
        if (t == 0) st_release_u64(a.word + (int64_t)buf * nblk + c, par | k);
    };

    const int lo0 = (int)max((int64_t)0, min((int64_t)nr, a.k0 - r0));
    int mycand = -1;
    {
        const unsigned long long k0key = argmax(0, lo0, false, 0.0, mycand);
        candidate_rcp(0, mycand);
        __syncthreads();
        publish(0, k0key, mycand);
    }
    for (int j = 0; j < kb; j++) {
        const int64_t g = a.k0 + j;
        const int buf = j & 1;
        const unsigned long long par = (unsigned long long)((j >> 1) & 1);
        // (1) the winner of column j: every thread polls at most one CTA's word per pass
        //     (relaxed loads issued together, one acquire fence once all have arrived)
        {
            unsigned long long bv = 0;
            int bc = INT_MAX;
            for (int q0 = 0; q0 < nblk; q0 += blockDim.x) {
                const int q = q0 + t;
                if (q < nblk) {
                    const unsigned long long *w = a.word + (int64_t)buf * nblk + q;
                    unsigned long long u = ld_relaxed_u64(w);
                    if ((u >> 63) != par) {
                        const unsigned long long t0 = global_ns();
                        while (((u = ld_relaxed_u64(w)) >> 63) != par) {
                            if (*(volatile int *)&a.bar->err || global_ns() - t0 > kWaitLimitNs) {
                                atomicExch(&a.bar->err, 1);
                                s_abort = 1;
                                break;
                            }
                        }
                    }
                    const unsigned long long val = u & 0x7fffffffffffffffull;
                    if (val > bv) {
                        bv = val;
                        bc = q;
                    }
                }
            }
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oc = __shfl_xor_sync(0xffffffffu, bc, o);
                if (ov > bv || (ov == bv && oc < bc)) {
                    bv = ov;
                    bc = oc;
                }
            }
            if (lane == 0) {
                red_w[warp] = bv;
                red_c[warp] = bc;
            }
            __syncthreads();
            if (t == 0) {
                for (int w = 1; w < (int)(blockDim.x >> 5); w++)
                    if (red_w[w] > red_w[0] || (red_w[w] == red_w[0] && red_c[w] < red_c[0])) {
                        red_w[0] = red_w[w];
                        red_c[0] = red_c[w];
                    }
                s_win = red_c[0];
            }
        }
        __syncthreads();
        if (s_abort) return;
        // no candidate anywhere (every |a| of the column NaN): row g stays, as the pivot
        const bool none = s_win == INT_MAX;
        const int own_g = (int)((g - a.k0) / rpc);
        const int win = none ? own_g : s_win;
        // (2) the pivot row with its reciprocal, and for the winner the old row g
        if (t <= kb) {
            if (none) s_piv[t] = t < kb ? __ldcg(a.diagbuf + buf * kb + t) : 0.0;
            else s_piv[t == kb ? kPanel : t] = __ldcg(a.rowbuf + ((int64_t)buf * nblk + win) * kRowBufLd +
                                                      (t == kb ? kPanel : t));
            if (win == c && t < kb) s_old[t] = __ldcg(a.diagbuf + buf * kb + t);
        }
        __syncthreads();
        // (3) the swap
        const int64_t p = (win == c) ? (none ? g : r0 + mycand) : -1;
        if (win == c && t == 0) a.ipiv[g] = (int32_t)p;
        if (t < kb) {
            if (win == c && p != g) P[(p - r0) * kb + t] = s_old[t];
            if (g >= r0 && g < r0 + nr) P[(g - r0) * kb + t] = s_piv[t];
        }
        const int lr1 = (int)max((int64_t)0, min((int64_t)nr, g + 1 - r0));  // first local row > g
        const double piv = s_piv[j];
        const bool ok = piv != 0.0 && isfinite(piv);
        if (!ok && t == 0) atomicCAS(&a.bar->info, 0, (int)(g + 1));
        // (3b) scale column j below g (rows > g are not touched by the swap's writes to row g;
        //      the winner's write to row p is by the same threads, t < kb, before their scaling)
        __syncthreads();
        if (ok) {
            const double rp = s_piv[kPanel];  // = 1 / piv, computed by the publisher
            for (int lr = lr1 + t; lr < nr; lr += blockDim.x) P[lr * kb + j] *= rp;
        }
        __syncthreads();
        if (j + 1 == kb) break;
        // (4) look-ahead: column j + 1 (updated on the way), the next candidate, its row and
        //     row g + 1, published
        int cand;
        const unsigned long long v = argmax(j + 1, lr1, ok, s_piv[j + 1], cand);
        candidate_rcp(j + 1, cand);
        const int lg1 = (g + 1 >= r0 && g + 1 < r0 + nr) ? (int)(g + 1 - r0) : -1;
        if (ok) {
            const int q = j + 2 + (t & 63);
            const int which = t >> 6;  // 0: the candidate row, 1: row g + 1
            const int lr = which == 0 ? cand : (lg1 != cand ? lg1 : -1);
            if (which < 2 && lr >= 0 && q < kb) P[lr * kb + q] = fma(-P[lr * kb + j], s_piv[q], P[lr * kb + q]);
        }
        __syncthreads();
        publish(j + 1, v, cand);
        // (5) the rest of the rank-1 update (columns > j + 1), beside the exchange
        if (ok) {
            const int q = t % kPanel, rg = t / kPanel;
            constexpr int kRowStep = 256 / kPanel;
            if (q > j + 1 && q < kb) {
                const double u = s_piv[q];
                for (int lr = lr1 + rg; lr < nr; lr += kRowStep)
                    if (lr != cand && lr != lg1) P[lr * kb + q] = fma(-P[lr * kb + j], u, P[lr * kb + q]);
            }
        }
        mycand = cand;
        __syncthreads();
    }
    for (int e = t; e < nr * kb; e += blockDim.x) {
        const int lr = e / kb, j = e - lr * kb;
        a.A[(r0 + lr) * a.ld + a.k0 + j] = P[e];
    }
}

// The panel's kb row interchanges (LAPACK laswp: for q = 0..kb-1 swap rows k0 + q and
// ipiv[k0 + q]) applied to the columns [c0, c1), and with TRSM also U12 = L11^-1 A12 (the
// unit lower L11 = A[k0:k0+kb, k0:k0+kb]) for the columns right of the panel.  Instead of
// kb dependent read-modify-write swaps per column, each CTA first works out in shared
// memory where every touched row's final content comes from (at most 2 kb rows: the panel
// rows and the pivot rows below them); then each thread gathers its column's touched rows
// with independent loads, solves, and writes them back.
constexpr int kSwapThreads = 128;
template <bool TRSM>
__global__ void __launch_bounds__(kSwapThreads) swap_trsm_kernel(double *A, int64_t ld, const int32_t *ipiv,
                                                                  int64_t k0, int kb, int64_t c0, int64_t c1) {
    __shared__ double L[TRSM ? kPanel : 1][kPanel + 1];
    __shared__ int64_t srow[2 * kPanel];   // slot -> row whose old content the slot's row receives
    __shared__ int64_t xrow[kPanel];       // extra slot kb + e -> its row (a pivot row below the panel)
    __shared__ int src[2 * kPanel];        // slot -> source slot, built by warp 0
    __shared__ int s_ne;
    extern __shared__ double E[];          // [extras][kSwapThreads]: old contents for the extra rows
    const int t = threadIdx.x;
    if (TRSM)
        for (int e = t; e < kb * kb; e += blockDim.x) {
            const int r = e / kb, q = e - r * kb;
            L[r][q] = A[(k0 + r) * ld + k0 + q];
        }
    if (t < 32) {
        // slots 0..kb-1: rows k0..k0+kb-1; kb.. : pivot rows below the panel, in order of appearance
        for (int q = t; q < 2 * kPanel; q += 32) src[q] = q;
        int ne = 0;
        __syncwarp();
        for (int q = 0; q < kb; q++) {
            const int64_t p = ipiv[k0 + q];
            int b;
            if (p < k0 + kb) {
                b = (int)(p - k0);
            } else {
                const bool hit0 = t < ne && xrow[t] == p, hit1 = t + 32 < ne && xrow[t + 32] == p;
                const unsigned m0 = __ballot_sync(0xffffffffu, hit0), m1 = __ballot_sync(0xffffffffu, hit1);
                if (m0) b = kb + __ffs(m0) - 1;
                else if (m1) b = kb + 32 + __ffs(m1) - 1;
                else {
                    if (t == 0) xrow[ne] = p;
                    b = kb + ne;
                    ne++;
                }
            }
            if (t == 0 && b != q) {
                const int tmp = src[q];
                src[q] = src[b];
                src[b] = tmp;
            }
            __syncwarp();
        }
        if (t == 0) s_ne = ne;
        __syncwarp();
        for (int sl = t; sl < kb + ne; sl += 32) {
            const int so = src[sl];
            srow[sl] = so < kb ? k0 + so : xrow[so - kb];
        }
    }
    __syncthreads();
    const int ne = s_ne;
    const int64_t c = c0 + (int64_t)blockIdx.x * blockDim.x + t;
    if (c >= c1) return;
    double x[kPanel];
#pragma unroll
    for (int q = 0; q < kPanel; q++)
        if (q < kb) x[q] = A[srow[q] * ld + c];
    for (int e = 0; e < ne; e++) E[e * kSwapThreads + t] = A[srow[kb + e] * ld + c];
    if (TRSM) {
#pragma unroll
        for (int r = 0; r < kPanel; r++) {
            double v = x[r];
#pragma unroll
            for (int q = 0; q < r; q++) v = fma(-L[r][q], x[q], v);
            x[r] = v;
        }
    }
#pragma unroll
    for (int q = 0; q < kPanel; q++)
        if (q < kb) A[(k0 + q) * ld + c] = x[q];
    for (int e = 0; e < ne; e++) A[xrow[e] * ld + c] = E[e * kSwapThreads + t];
}

// row swaps of rows k0 .. k0+kb-1 on columns [c0, c1)
__global__ void laswp_kernel(double *A, int64_t ld, const int32_t *ipiv, int64_t k0, int kb, int64_t c0, int64_t c1) {
    const int64_t c = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= c1) return;
    for (int q = 0; q < kb; q++) {
        const int64_t r = k0 + q, p = ipiv[r];
        if (p != r) {
            const double t = A[r * ld + c];
            A[r * ld + c] = A[p * ld + c];
            A[p * ld + c] = t;
        }
    }
}

// U12 = L11^-1 A12 (unit lower L11 = A[k0:k0+64, k0:k0+64]), thread per column;
// the column lives in registers (the panel width is always kPanel here)
__global__ void __launch_bounds__(128) trsm_f64_kernel(double *A, int64_t ld, int64_t k0, int64_t c0, int64_t c1) {
    __shared__ double L[kPanel][kPanel + 1];
    for (int e = threadIdx.x; e < kPanel * kPanel; e += blockDim.x) {
        const int r = e / kPanel, q = e - r * kPanel;
        L[r][q] = A[(k0 + r) * ld + k0 + q];
    }
    const int64_t c = c0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    __syncthreads();
    if (c >= c1) return;
    double x[kPanel];
#pragma unroll
    for (int r = 0; r < kPanel; r++) {
        double v = A[(k0 + r) * ld + c];
#pragma unroll
        for (int q = 0; q < r; q++) v = fma(-L[r][q], x[q], v);
        x[r] = v;
    }
#pragma unroll
    for (int r = 0; r < kPanel; r++) A[(k0 + r) * ld + c] = x[r];
}

// C (m x nc) -= L (m x kb) * U (kb x nc); FP64, 64x64 tiles, 4x4 per thread,
// K in chunks of 16
constexpr int DG_BK = 16;
__global__ void __launch_bounds__(256) dgemm_update_kernel(double *C, const double *Lp, const double *Up, int64_t ld,
                                                           int64_t m, int64_t nc, int kb) {
    __shared__ double As[DG_BK][64];  // As[k][row]
    __shared__ double Bs[DG_BK][64];  // Bs[k][col]
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t row0 = (int64_t)blockIdx.y * 64, col0 = (int64_t)blockIdx.x * 64;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < kb; k0 += DG_BK) {
        for (int e = threadIdx.x; e < 64 * DG_BK; e += 256) {
            const int r = e / DG_BK, k = e - r * DG_BK;
            As[k][r] = (row0 + r < m && k0 + k < kb) ? Lp[(row0 + r) * ld + k0 + k] : 0.0;
            const int k2 = e >> 6, cc = e & 63;
            Bs[k2][cc] = (col0 + cc < nc && k0 + k2 < kb) ? Up[(int64_t)(k0 + k2) * ld + col0 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < DG_BK; k++) {
            double av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) av[i] = As[k][ty * 4 + i];
#pragma unroll
            for (int j = 0; j < 4; j++) bv[j] = Bs[k][tx * 4 + j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int64_t r = row0 + ty * 4 + i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int64_t cc = col0 + tx * 4 + j;
            if (cc < nc) C[r * ld + cc] -= acc[i][j];
        }
    }
}

// ---- FP64 triangular solves (getrs) ------------------------------------------------
// Row interchanges in LAPACK order (swap rows r and ipiv[r] for r = 0, 1, ...).
// One CTA per right-hand side column; the column sits in shared memory while one
// thread applies the swaps (they compose, so they are sequential), then goes back.
constexpr int kPivSmemMax = 24576;  // doubles (192 KB)
__global__ void __launch_bounds__(256) apply_pivots_smem_kernel(double *B, int64_t ldb, const int32_t *ipiv,
                                                                int64_t n) {
    extern __shared__ double col[];
    const int64_t c = blockIdx.x;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) col[r] = B[r * ldb + c];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int64_t r = 0; r < n; r++) {
            const int64_t p = ipiv[r];
            if (p != r) {
                const double t = col[r];
                col[r] = col[p];
                col[p] = t;
            }
        }
    }
    __syncthreads();
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) B[r * ldb + c] = col[r];
}
// the same for columns too long for shared memory (one thread per column, global memory)
__global__ void apply_pivots_kernel(double *B, int64_t ldb, int64_t nrhs, const int32_t *ipiv, int64_t n) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nrhs) return;
    for (int64_t r = 0; r < n; r++) {
        const int64_t p = ipiv[r];
        if (p != r) {
            const double t = B[r * ldb + c];
            B[r * ldb + c] = B[p * ldb + c];
            B[p * ldb + c] = t;
        }
    }
}

// solve the diagonal block [b0, b0+bs) (bs <= 64) in place, lower unit or upper, for
// right-hand side column blockIdx.x: the block goes to shared memory (coalesced), then
// a column-oriented substitution with one thread per row and one barrier per column
template <bool UPPER>
__global__ void __launch_bounds__(64) trsv_block_kernel(const double *LU, int64_t ld, double *B, int64_t ldb,
                                                        int64_t nrhs, int64_t b0, int bs) {
    __shared__ double T[64][65];
    __shared__ double x[64];
    const int64_t c = blockIdx.x;
    const int r = threadIdx.x;
    for (int e = r; e < bs * bs; e += 64) {
        const int i = e / bs, q = e - i * bs;
        T[i][q] = LU[(b0 + i) * ld + b0 + q];
    }
    double v = r < bs ? B[(b0 + r) * ldb + c] : 0.0;
    __syncthreads();
    if (!UPPER) {
        for (int q = 0; q < bs; q++) {
            if (r == q) x[q] = v;
            __syncthreads();
            if (r > q) v = fma(-T[r][q], x[q], v);
        }
    } else {
        for (int q = bs - 1; q >= 0; q--) {
            if (r == q) {
                v = v / T[q][q];
                x[q] = v;
            }
            __syncthreads();
            if (r < q) v = fma(-T[r][q], x[q], v);
        }
    }
    if (r < bs) B[(b0 + r) * ldb + c] = v;
}

// B[rows r in [r0, r1)] -= LU[r, b0:b0+bs] * B[b0:b0+bs]; warp per (row, rhs)
__global__ void trsv_update_kernel(const double *LU, int64_t ld, double *B, int64_t ldb, int64_t nrhs, int64_t b0,
                                   int bs, int64_t r0, int64_t r1) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int64_t rows = r1 - r0;
    if (w >= rows * nrhs) return;
    const int64_t r = r0 + w / nrhs, c = w % nrhs;
    double acc = 0.0;
    for (int q = lane; q < bs; q += 32) acc = fma(LU[r * ld + b0 + q], B[(b0 + q) * ldb + c], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) B[r * ldb + c] -= acc;
}

// ---- low precision (FP32) no-pivot LU ----------------------------------------------
// One CTA (16 warps) factors the nb x nb diagonal block (nb <= 128, padded with
// the identity to 128) in shared memory, in 32 x 32 sub-blocks, and builds the
// inverses of its L and U factors alongside (they precondition the panels and
// the solves).  With X = inv(L) and Y = inv(U) started at zero, step s:
//   warp 0:  D[s][s] = L_ss U_ss (lane = row, the pivot row broadcast by warp
//            shuffles); the same sweep solves Y[s][s] U_ss = I row by row with
//            the broadcast pivot rows, and publishes each column of L_ss;
//   warp 4:  X[s][s] = inv(L_ss) column by column (lane = column), following
//            warp 0's published columns (bounded waits);
//   stage 1: U panel D[s][t] = X[s][s] D[s][t], L panel D[t][s] = D[t][s] Y[s][s]
//            (t > s); X[s][q] = X[s][s] X[s][q], Y[q][s] = Y[q][s] Y[s][s] (q < s);
//   stage 2: D[t][u] -= D[t][s] D[s][u] (t, u > s);
//            X[t][q] -= D[t][s] X[s][q] (t > s, q <= s);
//            Y[q][u] -= Y[q][s] D[s][u] (q <= s, u > s).
// Stage 2 looks ahead: warps 0 and 4 update D[s+1][s+1] alone and go on to step
// s + 1, while the 12 warps of the other three schedulers do the rest of stage 2
// and store the block row s of D and X and the block column s of Y (no later step
// changes them).  Warps 0 and 4 share scheduler 0 (warp w issues on scheduler
// w % 4): the latency-bound 32 x 32 factorization keeps a scheduler without
// block products.  The block products are bound by shared-memory bandwidth (one
// 16-byte load per lane per 8 FMA); measured per 128 x 128 block: 38.5 us with
// the pivot row through shared memory and stage 2 on two schedulers, 36.1 us
// with shuffles and three (bit-identical results).
// (X <- inv(L_s) X and Y <- Y inv(U_s) for the block-column / block-row factors
// L = L_0 L_1 L_2 L_3, U = U_3 U_2 U_1 U_0.)  Every stage-1/2 product is a
// 32 x 32 x 32 block product split into two warp tasks (16-row or 16-column
// halves, 4 x 4 outputs per lane, float4 operand loads); the row stride kLD
// keeps rows 16-byte aligned.
constexpr int kSB = 32;          // sub-block
constexpr int kNS = kNB / kSB;   // sub-blocks per side (4)
constexpr int kLD = kNB + 4;     // shared-memory row stride (floats)
constexpr size_t kDiagSmem = 3 * (size_t)kNB * kLD * sizeof(float);
constexpr int kPub = 4;                   // columns of L published per flag update
constexpr int kLinvWarp = 4;              // the inverse-of-L warp: scheduler 0, beside the LU warp
constexpr long long kDiagSpin = 1LL << 22;  // bounded wait of warp 1 on warp 0

__device__ __forceinline__ float *sblk(float *M, int i, int j) { return M + i * kSB * kLD + j * kSB; }
__device__ __forceinline__ const float *sblk(const float *M, int i, int j) { return M + i * kSB * kLD + j * kSB; }

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ int ld_volatile_s32(const int *p) { return *(const volatile int *)p; }

// Warp 0: row-per-lane LU of P (pivot row by shuffles from lane j) and, in the same sweep,
// Y = inv(U) by rows (Y U = I solved left to right with the pivot rows already broadcast);
// publishes column j of L (multipliers, zero on and above the diagonal) to Lc[j][0..32) for the
// inverse warp, kPub columns at a time.
__device__ __forceinline__ void lu32_fused(float *P, float *Yb, float *Lc, int *flag, int flag0, int lane, int row0,
                                           int nb, int64_t k0, int *info) {
    float a[kSB], y[kSB];
#pragma unroll
    for (int c4 = 0; c4 < kSB; c4 += 4) {
        const float4 v = *reinterpret_cast<const float4 *>(P + lane * kLD + c4);
        a[c4] = v.x, a[c4 + 1] = v.y, a[c4 + 2] = v.z, a[c4 + 3] = v.w;
        y[c4] = y[c4 + 1] = y[c4 + 2] = y[c4 + 3] = 0.0f;
    }
    unsigned bad = 0;
#pragma unroll
    for (int j = 0; j < kSB; j++) {
        const float piv = __shfl_sync(0xffffffffu, a[j], j);
        const bool ok = piv != 0.0f && isfinite(piv);
        bad |= (ok || row0 + j >= nb) ? 0u : (1u << j);
        const float rp = ok ? rcp_approx(piv) : 0.0f;
        // Y row `lane`: y[j] = (delta - sum_{k<j} Y_k U_kj) / U_jj, then the later sums
        const float yj = (((lane == j) ? 1.0f : 0.0f) - y[j]) * rp;
        y[j] = yj;
        const float l = lane > j ? a[j] * rp : 0.0f;
        if (lane > j) a[j] = l;
        Lc[j * kSB + lane] = l;
#pragma unroll
        for (int c = j + 1; c < kSB; c++) {
            const float u = __shfl_sync(0xffffffffu, a[c], j);  // pivot row j, column c
            a[c] = fmaf(-l, u, a[c]);
            y[c] = fmaf(yj, u, y[c]);
        }
        if (j % kPub == kPub - 1) {
            __syncwarp();
            if (lane == 0) {
                __threadfence_block();
                *(volatile int *)flag = flag0 + j + 1;
            }
        }
    }
    if (bad && lane == 0) atomicCAS(info, 0, (int)(k0 + row0 + __ffs(bad)));
#pragma unroll
    for (int c4 = 0; c4 < kSB; c4 += 4) {
        *reinterpret_cast<float4 *>(P + lane * kLD + c4) = make_float4(a[c4], a[c4 + 1], a[c4 + 2], a[c4 + 3]);
        *reinterpret_cast<float4 *>(Yb + lane * kLD + c4) = make_float4(y[c4], y[c4 + 1], y[c4 + 2], y[c4 + 3]);
    }
}

// Warp 4: X = inv(L) column `lane`, right-looking forward substitution over the published columns
// of L (waits, bounded, for each group of kPub; on a timeout raises info[1] and stops).
__device__ __forceinline__ void linv32_follow(const float *Lc, float *Xb, const int *flag, int flag0, int lane,
                                              int *info) {
    float x[kSB];
#pragma unroll
    for (int i = 0; i < kSB; i++) x[i] = (i == lane) ? 1.0f : 0.0f;
    bool alive = true;
#pragma unroll
    for (int k = 0; k < kSB; k++) {
        if (k % kPub == 0) {
            long long it = 0;
            while (alive && ld_volatile_s32(flag) < flag0 + k + kPub) {
                if (++it > kDiagSpin) {
                    if (lane == 0) atomicExch(info + 1, 1);
                    alive = false;
                }
            }
            __syncwarp();
            __threadfence_block();
        }
#pragma unroll
        for (int i4 = (k + 1) & ~3; i4 < kSB; i4 += 4) {
            const float4 v = *reinterpret_cast<const float4 *>(Lc + k * kSB + i4);
            if (i4 > k) x[i4] = fmaf(-v.x, x[k], x[i4]);
            if (i4 + 1 > k) x[i4 + 1] = fmaf(-v.y, x[k], x[i4 + 1]);
            if (i4 + 2 > k) x[i4 + 2] = fmaf(-v.z, x[k], x[i4 + 2]);
            if (i4 + 3 > k) x[i4 + 3] = fmaf(-v.w, x[k], x[i4 + 3]);
        }
    }
#pragma unroll
    for (int i = 0; i < kSB; i++) Xb[i * kLD + lane] = x[i];
}

// One warp: C (=|-=) A B over k = 32, C of (128 / CG) rows x (4 CG) columns, 4 x 4
// per lane.  Lane group g = lane / CG owns rows g + G i (G = 32 / CG groups), so the
// 16-byte A loads of one instruction fall in distinct bank groups (row stride kLD).
// C may alias A when CG = 8 (row halves read only their own rows of A) or B when
// CG = 4 (column halves read only their own columns of B): all operands are read
// before the first store.
template <int CG, bool SUB>
__device__ __forceinline__ void warp_mm(const float *A, const float *B, float *C, int lane) {
    constexpr int G = 32 / CG;
    const int g = lane / CG, c0 = (lane % CG) * 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (SUB) {
            const float4 v = *reinterpret_cast<const float4 *>(C + (g + G * i) * kLD + c0);
            acc[i][0] = v.x, acc[i][1] = v.y, acc[i][2] = v.z, acc[i][3] = v.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
        }
    }
#pragma unroll 2
    for (int k = 0; k < kSB; k += 4) {
        float a[4][4], b[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const float4 v = *reinterpret_cast<const float4 *>(A + (g + G * i) * kLD + k);
            a[i][0] = SUB ? -v.x : v.x, a[i][1] = SUB ? -v.y : v.y, a[i][2] = SUB ? -v.z : v.z,
            a[i][3] = SUB ? -v.w : v.w;
            const float4 w = *reinterpret_cast<const float4 *>(B + (k + i) * kLD + c0);
            b[i][0] = w.x, b[i][1] = w.y, b[i][2] = w.z, b[i][3] = w.w;
        }
#pragma unroll
        for (int kk = 0; kk < 4; kk++)
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i][kk], b[kk][j], acc[i][j]);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 4; i++)
        *reinterpret_cast<float4 *>(C + (g + G * i) * kLD + c0) =
            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    __syncwarp();
}

// store the finished parts of step s: rows [32s, 32s + 32) of the factored block and of inv(L),
// columns [32s, 32s + 32) of inv(U) (and the same rows of its transpose); threads t0 .. t0 + nt
__device__ __forceinline__ void diag_store_step(int s, const float *D, const float *X, const float *Y, float *A,
                                                int64_t ld, int64_t k0, int nb, bool v4, float *Linv, float *Uinv,
                                                float *UinvT, int t, int nt) {
    const int r0 = s * kSB;
    for (int e = t; e < kSB * kNB / 4; e += nt) {  // 32 rows x 32 float4
        const int r = r0 + (e >> 5), c4 = (e & 31) * 4;
        const float4 d = *reinterpret_cast<const float4 *>(D + r * kLD + c4);
        if (v4) {
            *reinterpret_cast<float4 *>(A + (k0 + r) * ld + k0 + c4) = d;
        } else if (r < nb) {
            const float w[4] = {d.x, d.y, d.z, d.w};
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (c4 + q < nb) A[(k0 + r) * ld + k0 + c4 + q] = w[q];
        }
        *reinterpret_cast<float4 *>(Linv + r * kNB + c4) = *reinterpret_cast<const float4 *>(X + r * kLD + c4);
    }
    for (int e = t; e < kNB * kSB / 4; e += nt) {  // 128 rows x 8 float4 of column block s
        const int r = e >> 3, c4 = r0 + (e & 7) * 4;
        *reinterpret_cast<float4 *>(Uinv + r * kNB + c4) = *reinterpret_cast<const float4 *>(Y + r * kLD + c4);
    }
    if (UinvT)
        for (int e = t; e < kSB * kNB; e += nt) {  // rows r0 .. r0 + 32 of the transpose
            const int c = r0 + (e >> 7), r = e & (kNB - 1);
            UinvT[c * kNB + r] = Y[r * kLD + c];
        }
}

// One CTA per system of a batch: system z = blockIdx.x at A + z sA, Linv / Uinv + z sD,
// UinvT + z sT, its flags at info + 2 z.
__global__ void __launch_bounds__(512) diag_lowp_kernel(float *A, int64_t ld, int64_t k0, int nb, float *Linv,
                                                        float *Uinv, float *UinvT, int *info, int64_t sA, int64_t sD,
                                                        int64_t sT) {
    extern __shared__ __align__(16) float sm[];
    {
        const int64_t z = blockIdx.x;
        A += z * sA, Linv += z * sD, Uinv += z * sD, info += 2 * z;
        if (UinvT) UinvT += z * sT;
    }
    float *D = sm, *X = sm + kNB * kLD, *Y = sm + 2 * kNB * kLD;
    __shared__ __align__(16) float Lc[kSB * kSB];
    __shared__ int flag;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nthr = blockDim.x, nwarp = nthr >> 5;
    if (tid == 0) flag = 0;
    const bool v4 = nb == kNB && (((uintptr_t)(A + k0 * ld + k0)) & 15) == 0;
    {
        const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 buf[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int e = tid + u * 512, r = e >> 5, c4 = (e & 31) * 4;
            if (v4) {
                buf[u] = __ldg(reinterpret_cast<const float4 *>(A + (k0 + r) * ld + k0 + c4));
            } else {
                float w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int c = c4 + q;
                    w[q] = (r < nb && c < nb) ? A[(k0 + r) * ld + k0 + c] : (r == c ? 1.0f : 0.0f);
                }
                buf[u] = make_float4(w[0], w[1], w[2], w[3]);
            }
        }
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const int e = tid + u * 512, r = e >> 5, c4 = (e & 31) * 4;
            *reinterpret_cast<float4 *>(D + r * kLD + c4) = buf[u];
            *reinterpret_cast<float4 *>(X + r * kLD + c4) = z4;
            *reinterpret_cast<float4 *>(Y + r * kLD + c4) = z4;
        }
    }
    __syncthreads();
    for (int s = 0; s < kNS; s++) {
        const int m = kNS - 1 - s;
        // factor D[s][s] (warp 0) and invert L_ss (warp kLinvWarp); the other warps finish stage 2 of s - 1
        if (warp == 0) lu32_fused(sblk(D, s, s), sblk(Y, s, s), Lc, &flag, s * kSB, lane, s * kSB, nb, k0, info);
        else if (warp == kLinvWarp) linv32_follow(Lc, sblk(X, s, s), &flag, s * kSB, lane, info);
        __syncthreads();
        for (int t = warp; t < 2 * (2 * m + 2 * s); t += nwarp) {
            const int b = t >> 1, h = (t & 1) * 16;
            if (b < m) {
                float *C = sblk(D, s, s + 1 + b) + h;
                warp_mm<4, false>(sblk(X, s, s), C, C, lane);
            } else if (b < 2 * m) {
                float *C = sblk(D, s + 1 + (b - m), s) + h * kLD;
                warp_mm<8, false>(C, sblk(Y, s, s), C, lane);
            } else if (b < 2 * m + s) {
                float *C = sblk(X, s, b - 2 * m) + h;
                warp_mm<4, false>(sblk(X, s, s), C, C, lane);
            } else {
                float *C = sblk(Y, b - 2 * m - s, s) + h * kLD;
                warp_mm<8, false>(C, sblk(Y, s, s), C, lane);
            }
        }
        __syncthreads();
        if (m == 0) break;
        if (warp == 0 || warp == kLinvWarp) {
            // look-ahead: the block the next factorization needs, D[s+1][s+1] -= D[s+1][s] D[s][s+1]
            // (a 16-row half each), then on to step s + 1 while the other warps finish stage 2
            const int h = warp == 0 ? 0 : 16;
            warp_mm<8, true>(sblk(D, s + 1, s) + h * kLD, sblk(D, s, s + 1), sblk(D, s + 1, s + 1) + h * kLD, lane);
            asm volatile("bar.sync 1, 64;" ::: "memory");
        } else if ((warp & 3) != 0) {
            // the rest of stage 2 (m^2 - 1 blocks of D, m (s + 1) of X and of Y), then the stores of
            // step s, on the 12 warps of the three schedulers that warps 0 and kLinvWarp do not use
            const int w12 = (warp >> 2) * 3 + (warp & 3) - 1;
            const int nD = m * m - 1, nX = m * (s + 1);
            for (int t = w12; t < 2 * (nD + 2 * nX); t += 12) {
                const int b = t >> 1, h = (t & 1) * 16;
                if (b < nD) {
                    const int i = (b + 1) / m, j = (b + 1) - ((b + 1) / m) * m;
                    warp_mm<8, true>(sblk(D, s + 1 + i, s) + h * kLD, sblk(D, s, s + 1 + j),
                                     sblk(D, s + 1 + i, s + 1 + j) + h * kLD, lane);
                } else if (b < nD + nX) {
                    const int i = (b - nD) / (s + 1), q = (b - nD) % (s + 1);
                    warp_mm<8, true>(sblk(D, s + 1 + i, s) + h * kLD, sblk(X, s, q), sblk(X, s + 1 + i, q) + h * kLD,
                                     lane);
                } else {
                    const int q = (b - nD - nX) / m, j = (b - nD - nX) % m;
                    warp_mm<8, true>(sblk(Y, q, s) + h * kLD, sblk(D, s, s + 1 + j), sblk(Y, q, s + 1 + j) + h * kLD,
                                     lane);
                }
            }
            diag_store_step(s, D, X, Y, A, ld, k0, nb, v4, Linv, Uinv, UinvT, w12 * 32 + lane, 12 * 32);
        }
    }
    diag_store_step(kNS - 1, D, X, Y, A, ld, k0, nb, v4, Linv, Uinv, UinvT, tid, nthr);
}

// Panels of one LU step, in place, in one launch (CTA x < ntu: U tiles, else L tiles):
//   U12[:, 32-col tile] = Linv (128 x 128) * A12[:, tile]  (all 128 rows per CTA; also
//                         written transposed into Ut (nr rows of 128, row stride ldu, K-major)
//                         for the tensor cores)
//   L21[32-row tile, :] = A21[tile, :] * Uinv (128 x 128)  (all 128 columns per CTA)
// Each CTA reads its whole input tile before writing it back, so in place is safe.
__global__ void __launch_bounds__(256) lowp_panel_kernel(float *A, int64_t ld, int64_t k0, int64_t nr,
                                                         const float *Linv, const float *Uinv, float *Ut, int64_t ldu,
                                                         int ntu) {
    __shared__ float tile[kNB][33];  // U: [row][col]; L: stored as [col][row]
    const int64_t c0 = k0 + kNB;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if ((int)blockIdx.x < ntu) {
        const int64_t j0 = (int64_t)blockIdx.x * 32;
        const int cols = (int)min((int64_t)32, nr - j0);
        for (int e = t; e < kNB * 32; e += 256) {
            const int r = e >> 5, c = e & 31;
            tile[r][c] = c < cols ? A[(k0 + r) * ld + c0 + j0 + c] : 0.0f;
        }
        __syncthreads();
        float acc[16];
#pragma unroll
        for (int k = 0; k < 16; k++) acc[k] = 0.0f;
        for (int q = 0; q < kNB; q++) {
            const float b = tile[q][lane];
#pragma unroll
            for (int k = 0; k < 16; k++) acc[k] = fmaf(Linv[(w + 8 * k) * kNB + q], b, acc[k]);
        }
        if (lane < cols) {
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const int r = w + 8 * k;
                A[(k0 + r) * ld + c0 + j0 + lane] = acc[k];
                Ut[(j0 + lane) * ldu + r] = acc[k];
            }
        }
    } else {
        const int64_t i0 = (int64_t)(blockIdx.x - ntu) * 32;
        const int rows = (int)min((int64_t)32, nr - i0);
        for (int e = t; e < 32 * kNB; e += 256) {
            const int r = e >> 7, c = e & (kNB - 1);
            tile[c][r] = r < rows ? A[(c0 + i0 + r) * ld + k0 + c] : 0.0f;
        }
        __syncthreads();
        // thread: column c = t % 128, rows r = t / 128 + 2 k
        const int c = t & (kNB - 1), rb = t >> 7;
        float acc[16];
#pragma unroll
        for (int k = 0; k < 16; k++) acc[k] = 0.0f;
        for (int q = 0; q < kNB; q++) {
            const float u = Uinv[q * kNB + c];
#pragma unroll
            for (int k = 0; k < 16; k++) acc[k] = fmaf(tile[q][rb + 2 * k], u, acc[k]);
        }
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const int r = rb + 2 * k;
            if (r < rows) A[(c0 + i0 + r) * ld + k0 + c] = acc[k];
        }
    }
}

// C = alpha A B + beta C (row-major FP32, CUDA cores); 128x128 tiles, 8x8 per thread
constexpr int SG_BM = 128, SG_BN = 128, SG_BK = 8;
__global__ void __launch_bounds__(256) sgemm_kernel(int64_t M, int64_t N, int64_t K, float alpha, const float *A,
                                                    int64_t lda, const float *B, int64_t ldb, float beta, float *C,
                                                    int64_t ldc) {
    __shared__ float As[SG_BK][SG_BM];
    __shared__ float Bs[SG_BK][SG_BN];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int64_t row0 = (int64_t)blockIdx.y * SG_BM, col0 = (int64_t)blockIdx.x * SG_BN;
    float acc[8][8] = {};
    for (int64_t k0 = 0; k0 < K; k0 += SG_BK) {
        for (int e = threadIdx.x; e < SG_BM * SG_BK; e += 256) {
            const int r = e / SG_BK, k = e % SG_BK;
            As[k][r] = (row0 + r < M && k0 + k < K) ? A[(row0 + r) * lda + k0 + k] : 0.0f;
            const int k2 = e / SG_BN, cc = e % SG_BN;
            Bs[k2][cc] = (k0 + k2 < K && col0 + cc < N) ? B[(k0 + k2) * ldb + col0 + cc] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SG_BK; k++) {
            float av[8], bv[8];
#pragma unroll
            for (int i = 0; i < 8; i++) av[i] = As[k][ty * 8 + i];
#pragma unroll
            for (int j = 0; j < 8; j++) bv[j] = Bs[k][tx * 8 + j];
#pragma unroll
            for (int i = 0; i < 8; i++)
#pragma unroll
                for (int j = 0; j < 8; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int64_t r = row0 + ty * 8 + i;
        if (r >= M) continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int64_t c = col0 + tx * 8 + j;
            if (c < N) C[r * ldc + c] = alpha * acc[i][j] + (beta == 0.0f ? 0.0f : beta * C[r * ldc + c]);
        }
    }
}

__global__ void copy2d_f32_kernel(const float *src, int64_t lds, float *dst, int64_t ldd, int64_t rows, int64_t cols) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t r = blockIdx.y; r < rows; r += gridDim.y)
        if (c < cols) dst[r * ldd + c] = src[r * lds + c];
}

// dst (cols x rows, ldd) = src^T (rows x cols, lds); system blockIdx.z at src + z ss, dst + z sd
__global__ void transpose_f32_kernel(const float *src, int64_t lds, float *dst, int64_t ldd, int64_t rows,
                                     int64_t cols, int64_t ss, int64_t sd) {
    __shared__ float t[32][33];
    src += blockIdx.z * ss, dst += blockIdx.z * sd;
    const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        t[i][threadIdx.x] = (r < rows && c < cols) ? src[r * lds + c] : 0.0f;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (c < cols && r < rows) dst[c * ldd + r] = t[threadIdx.x][i];
    }
}

// tensor-core update (tc_gemm.cu): C (m x nc, ldc) -= Lp (m x K, ldl) * Ut^T (nc x K, ldu), K % 128 == 0,
// for one system or a batch of them (TcBatch)
size_t tc_update_bytes(int64_t m, int64_t nc, int64_t K, int mode, int nb = 1);
int tc_update(float *C, int64_t ldc, const float *Lp, int64_t ldl, const float *Ut, int64_t ldu, int64_t m,
              int64_t nc, int64_t K, int mode, void *work, size_t work_bytes, cudaStream_t st, int *err_dev,
              bool store = false, int tile = 0, int max_ctas = 0, const TcBatch &bt = TcBatch{});
// the BF16 update from operands already rounded to BF16 (La, Ub: K-major __nv_bfloat16)
int tc_update_bf16(float *C, int64_t ldc, const void *La, int64_t ldl, const void *Ub, int64_t ldu, int64_t m,
                   int64_t nc, int64_t K, void *work, size_t work_bytes, cudaStream_t st, int *err_dev, int tile,
                   int max_ctas, const TcBatch &bt);

// BF16 copies of one step's finished panels for the BF16 trailing updates: blockIdx.y = 0
// rounds the L panel (nr rows x 128, row stride lda) into Lb, 1 the K-major U panel (nr rows
// x 128, row stride ldu) into Ub (row stride ldb); system blockIdx.z at + z (sA, sU, sB).
__global__ void __launch_bounds__(256) panel_bf16_kernel(const float *L21, int64_t lda, const float *Ut, int64_t ldu,
                                                         __nv_bfloat16 *Lb, __nv_bfloat16 *Ub, int64_t ldb,
                                                         int64_t nr, int64_t sA, int64_t sU, int64_t sB) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, r = i >> 5;
    if (r >= nr) return;
    const int c4 = (int)(i & 31) * 4;
    const int64_t z = blockIdx.z;
    const float *src = blockIdx.y == 0 ? L21 + z * sA + r * lda : Ut + z * sU + r * ldu;
    __nv_bfloat16 *dst = (blockIdx.y == 0 ? Lb : Ub) + z * sB + r * ldb;
    const float4 v = *reinterpret_cast<const float4 *>(src + c4);
    __nv_bfloat162 lo = __floats2bfloat162_rn(v.x, v.y), hi = __floats2bfloat162_rn(v.z, v.w);
    uint2 w;
    w.x = *reinterpret_cast<uint32_t *>(&lo);
    w.y = *reinterpret_cast<uint32_t *>(&hi);
    *reinterpret_cast<uint2 *>(dst + c4) = w;
}

static int sgemm(cudaStream_t st, int64_t M, int64_t N, int64_t K, float alpha, const float *A, int64_t lda,
                 const float *B, int64_t ldb, float beta, float *C, int64_t ldc) {
    if (M == 0 || N == 0) return FLG_OK;
    dim3 grid((unsigned)ceil_div(N, SG_BN), (unsigned)ceil_div(M, SG_BM));
    sgemm_kernel<<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

static int copy2d(cudaStream_t st, const float *src, int64_t lds, float *dst, int64_t ldd, int64_t rows, int64_t cols) {
    if (rows == 0 || cols == 0) return FLG_OK;
    dim3 grid((unsigned)ceil_div(cols, 256), (unsigned)std::min<int64_t>(rows, 65535));
    copy2d_f32_kernel<<<grid, 256, 0, st>>>(src, lds, dst, ldd, rows, cols);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

// ---- low precision triangular solve with the diagonal-block inverses ------------------
// x = U^-1 L^-1 b for one right-hand side, FP32 factors, as a dataflow over the 128-row
// blocks in ONE cooperative launch of G CTAs.  CTA c owns the q consecutive blocks
// [c q, c q + q) (q <= kApplyQ).  In "pass order" -- the forward pass by increasing block,
// the backward pass by decreasing block -- block p needs every earlier block p' < p:
//   forward   y_i = Linv_i (b_i - sum_{j<i} L_ij y_j)
//   backward  x_i = Uinv_i (y_i - sum_{j>i} U_ij x_j).
// A CTA accumulates the contributions of the blocks before its chunk as their owners
// publish them, then runs through its own chunk locally: each finished block goes straight
// from shared memory into the later blocks of the chunk, so only one result in q crosses
// between SMs (through L2) on the critical chain.
//   * One producer thread streams the 128 x 128 FP32 slices in the order they are used
//     (for each earlier source block, its slice for every own block; for each own block,
//     its inverse, then its slices for the later own blocks) by TMA (cp.async.bulk.tensor,
//     64 KB each) into a 3-stage shared-memory ring guarded by mbarriers; rows and
//     columns outside the matrix arrive as zeros.
//   * Eight consumer warps own 16 rows of every block; lane l multiplies columns
//     4l..4l+3 of its rows (one conflict-free 16-byte load per row) by its float4 of the
//     source block and keeps 16 running partial sums per own block; finishing a block
//     reduce-scatters them over the lanes (16 shuffles).
//   * Publication is the data itself: y and x start filled with an all-ones bit pattern
//     (a NaN that FP32 arithmetic never produces; results are stored canonicalized),
//     values are stored with st.relaxed.gpu and consumers poll their four elements with
//     ld.relaxed.gpu (bounded) -- no flag, no fence.  Every wait is on a block earlier in
//     the global order (forward, then backward) and all CTAs are resident, so the order
//     always advances.
// Each block's sum runs in one CTA in a fixed order (by source block), so the result does
// not depend on G.
constexpr int kApplyConsumers = 8;                         // warps
constexpr int kApplyThreads = (kApplyConsumers + 1) * 32;  // + the producer warp
constexpr int kApplyStages = 3;
constexpr int kApplyQ = 4;                  // at most this many blocks per CTA
constexpr int kSliceBytes = kNB * kNB * 4;  // 64 KB
constexpr size_t kApplySmem = (size_t)kApplyStages * kSliceBytes + 1024;
constexpr unsigned kUnset = 0xffffffffu;

struct ApplyArgs {
    int64_t n;
    int q;           // blocks per CTA
    const float *b;  // right-hand side (FP32, n)
    float *y, *x;    // forward / backward results (n), preset to kUnset
    int *err;        // a wait ran out
};

__device__ __forceinline__ void st_relaxed_f32(float *p, float v) {
    unsigned u = __float_as_uint(v);
    if (u == kUnset) u = 0x7fffffffu;  // keep the sentinel unique
    asm volatile("st.relaxed.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(u) : "memory");
}
__device__ __forceinline__ void tma_load_box(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive1(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// the published float4 of a block (elements e .. e+3, those < n; zeros beyond n): the four
// loads are issued together, then those still unset are polled together until published
__device__ __forceinline__ bool fetch4(const float *v, int64_t e, int64_t n, float4 &out, int *err) {
    const int cnt = (int)max((int64_t)0, min((int64_t)4, n - e));
    unsigned u[4];
#pragma unroll
    for (int k = 0; k < 4; k++) u[k] = k < cnt ? ld_relaxed_u32(v + e + k) : 0u;
    if (!wait_published4(reinterpret_cast<const unsigned *>(v + e), cnt, kUnset, u, kWaitLimitNs, err)) return false;
    out = make_float4(__uint_as_float(u[0]), __uint_as_float(u[1]), __uint_as_float(u[2]), __uint_as_float(u[3]));
    return true;
}

// sum of acc[0..15] over the 32 lanes, scattered: lanes 2r and 2r + 1 end with row r's total
__device__ __forceinline__ float reduce_scatter16(float (&acc)[16], int lane) {
    float a8[8], a4[4], a2[2];
    const bool h4 = lane & 16, h3 = lane & 8, h2 = lane & 4, h1 = lane & 2;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const float send = h4 ? acc[k] : acc[8 + k];
        const float keep = h4 ? acc[8 + k] : acc[k];
        a8[k] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float send = h3 ? a8[k] : a8[4 + k];
        const float keep = h3 ? a8[4 + k] : a8[k];
        a4[k] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float send = h2 ? a4[k] : a4[2 + k];
        const float keep = h2 ? a4[2 + k] : a4[k];
        a2[k] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    const float send = h1 ? a2[0] : a2[1];
    const float keep = h1 ? a2[1] : a2[0];
    const float a1 = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    return a1 + __shfl_xor_sync(0xffffffffu, a1, 1);
}

// acc[sel] += S (16 rows of this warp) . v, for a run-time sel < kApplyQ
__device__ __forceinline__ void slice_fma(float (&acc)[kApplyQ][16], int sel, const float *S, float4 v) {
#pragma unroll
    for (int q = 0; q < kApplyQ; q++)
        if (q == sel) {
#pragma unroll
            for (int r = 0; r < 16; r++) {
                const float4 w = *reinterpret_cast<const float4 *>(S + r * kNB);
                acc[q][r] = fmaf(w.x, v.x, acc[q][r]);
                acc[q][r] = fmaf(w.y, v.y, acc[q][r]);
                acc[q][r] = fmaf(w.z, v.z, acc[q][r]);
                acc[q][r] = fmaf(w.w, v.w, acc[q][r]);
            }
        }
}

__global__ void __launch_bounds__(kApplyThreads, 1)
    lowp_apply_kernel(const __grid_constant__ CUtensorMap mLU, const __grid_constant__ CUtensorMap mD, ApplyArgs a) {
    extern __shared__ __align__(1024) unsigned char apply_smem[];
    float *ring = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(apply_smem) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t full[kApplyStages], empty[kApplyStages];
    __shared__ __align__(16) float tvec[kNB], yvec[kNB];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    const int nblk = (int)ceil_div(a.n, kNB);
    const int c = blockIdx.x;
    const int b0 = c * a.q, b1 = min(nblk, b0 + a.q);  // own physical blocks [b0, b1)
    const int qc = max(0, b1 - b0);
    if (t == 0) {
        for (int q = 0; q < kApplyStages; q++) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], kApplyConsumers);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (qc == 0) return;
    // pass order: forward p = i, backward p = nblk - 1 - i; own pass-order blocks [p0, p0 + qc)
    auto blk = [&](bool fwd, int p) { return fwd ? p : nblk - 1 - p; };
    if (warp == kApplyConsumers) {
        if (lane == 0) {
            long long k = 0;  // slices issued
            bool ok = true;
            auto issue = [&](const CUtensorMap *m, int x, int y) {
                const int stg = (int)(k % kApplyStages);
                if (k >= kApplyStages &&
                    !mbar_wait(&empty[stg], (uint32_t)((k / kApplyStages - 1) & 1), a.err, kWaitLimitNs)) {
                    ok = false;
                    return;
                }
                mbar_arrive_expect(&full[stg], kSliceBytes);
                tma_load_box(ring + (size_t)stg * (kNB * kNB), m, &full[stg], x, y);
                k++;
            };
            for (int pass = 0; pass < 2 && ok; pass++) {
                const bool fwd = pass == 0;
                const int p0 = fwd ? b0 : nblk - b1;
                for (int pj = 0; pj < p0 + qc && ok; pj++) {
                    const int j = blk(fwd, pj);
                    if (pj >= p0) issue(&mD, 0, (fwd ? j : nblk + j) * kNB);
                    for (int p = max(p0, pj + 1); p < p0 + qc && ok; p++) issue(&mLU, j * kNB, blk(fwd, p) * kNB);
                }
            }
            // drain: every issued load has landed before the CTA may exit
            for (long long q = k > kApplyStages ? k - kApplyStages : 0; q < k; q++)
                mbar_drain(&full[q % kApplyStages], (uint32_t)((q / kApplyStages) & 1), a.err, kWaitLimitNs);
        }
        return;
    }
    // consumers.  After a wait has run out (a.err raised, possibly by another CTA) a warp
    // keeps the loop's structure -- every stage is still waited for (each wait now returns at
    // once) and released, and every named barrier is reached -- so the producer can stop and
    // drain and no warp waits on one that has left; the results are then discarded.
    long long k = 0;  // slices consumed
    bool dead = false;
    const int row0 = warp * 16;
    auto take = [&]() -> const float * {  // the next ring stage, this warp's rows and lane's columns
        const int stg = (int)(k % kApplyStages);
        dead = !__all_sync(0xffffffffu, !dead);
        if (!mbar_wait(&full[stg], (uint32_t)((k / kApplyStages) & 1), a.err, kWaitLimitNs)) dead = true;
        return ring + (size_t)stg * (kNB * kNB) + (size_t)row0 * kNB + 4 * lane;
    };
    auto release = [&]() {
        __syncwarp();
        if (lane == 0) mbar_arrive1(&empty[k % kApplyStages]);
        k++;
    };
    for (int pass = 0; pass < 2; pass++) {
        const bool fwd = pass == 0;
        float *out_v = fwd ? a.y : a.x;  // published into and consumed from
        const int p0 = fwd ? b0 : nblk - b1;
        float acc[kApplyQ][16];
#pragma unroll
        for (int q = 0; q < kApplyQ; q++)
#pragma unroll
            for (int r = 0; r < 16; r++) acc[q][r] = 0.0f;
        // this lane's right-hand side entries of the own blocks (lanes 2r, 2r + 1 hold row r)
        float rhs[kApplyQ];
#pragma unroll
        for (int q = 0; q < kApplyQ; q++) {
            rhs[q] = 0.0f;
            if (q < qc) {
                const int64_t e = (int64_t)blk(fwd, p0 + q) * kNB + row0 + (lane >> 1);
                if (e < a.n) rhs[q] = fwd ? a.b[e] : __uint_as_float(ld_relaxed_u32(a.y + e));
            }
        }
        for (int pj = 0; pj < p0 + qc; pj++) {
            const int j = blk(fwd, pj);
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (pj < p0) {
                // an earlier block, published by its owner
                if (!dead && !fetch4(out_v, (int64_t)j * kNB + 4 * lane, a.n, v, a.err)) dead = true;
            } else {
                // an own block: t = rhs - sums, then out_j = inverse . t, published and kept
                const int sel = pj - p0;
                float tmp[16];
                float rh = 0.0f;
#pragma unroll
                for (int q = 0; q < kApplyQ; q++)
                    if (q == sel) {
#pragma unroll
                        for (int r = 0; r < 16; r++) tmp[r] = acc[q][r];
                        rh = rhs[q];
                    }
                const float tot = reduce_scatter16(tmp, lane);
                if ((lane & 1) == 0) tvec[row0 + (lane >> 1)] = rh - tot;
                asm volatile("bar.sync 1, %0;" ::"r"(kApplyConsumers * 32) : "memory");
                const float4 tv = *reinterpret_cast<const float4 *>(tvec + 4 * lane);
#pragma unroll
                for (int r = 0; r < 16; r++) tmp[r] = 0.0f;
                const float *S = take();
#pragma unroll
                for (int r = 0; r < 16; r++) {
                    const float4 w = *reinterpret_cast<const float4 *>(S + r * kNB);
                    tmp[r] = fmaf(w.x, tv.x, tmp[r]);
                    tmp[r] = fmaf(w.y, tv.y, tmp[r]);
                    tmp[r] = fmaf(w.z, tv.z, tmp[r]);
                    tmp[r] = fmaf(w.w, tv.w, tmp[r]);
                }
                release();
                const float res = reduce_scatter16(tmp, lane);
                if ((lane & 1) == 0) {
                    const int r = row0 + (lane >> 1);
                    const int64_t e = (int64_t)j * kNB + r;
                    yvec[r] = e < a.n ? res : 0.0f;
                    if (e < a.n) st_relaxed_f32(out_v + e, res);
                }
                asm volatile("bar.sync 1, %0;" ::"r"(kApplyConsumers * 32) : "memory");
                v = *reinterpret_cast<const float4 *>(yvec + 4 * lane);
            }
            // (tvec and yvec are rewritten only after the next own block's first barrier, which
            // every warp reaches after its last read of them)
            for (int p = max(p0, pj + 1); p < p0 + qc; p++) {
                const float *S = take();
                slice_fma(acc, p - p0, S, v);
                release();
            }
        }
    }
}

__global__ void d2f_kernel(const double *a, float *b, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}
// FP32 solution back to FP64; NaN everywhere if a wait of the apply ran out
__global__ void f2d_kernel(const float *a, double *b, int64_t n, const int *err) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = *err ? __longlong_as_double(0x7ff8000000000000LL) : (double)a[i];
}

int make_box_map_f32(CUtensorMap *map, const float *base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                     int box_cols);

// blocks per CTA of the low-precision solve: 2 measured fastest on GB300 from n = 1,536 to
// 24,576 (1 hands every block between SMs; 3 and 4 lengthen each CTA's slice stream)
constexpr int kApplyQDefault = 2;

size_t lu_solve_lowp_bytes(int64_t n) {
    CountingArena c;
    c.take<float>(n);
    c.take<float>(2 * n);  // y, x: one sentinel fill
    c.take<int>(1);
    return c.bytes();
}

// the kernel attributes of the solve, set once (before any graph capture that includes it)
int lu_solve_lowp_prepare() {
    static bool attr_set = false;
    if (!attr_set) {
        FLG_CUDA(cudaFuncSetAttribute(lowp_apply_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kApplySmem));
        attr_set = true;
    }
    return FLG_OK;
}

int lu_solve_lowp_apply(int64_t n, const float *LU, int64_t ld, const float *dinv, const double *b, double *x,
                        void *work, size_t work_bytes, cudaStream_t st) {
    FLG_REQUIRE(ld % 4 == 0 && ((uintptr_t)LU & 15) == 0, "LU rows must be 16-byte aligned (ld % 4 == 0)");
    Arena ar(work, work_bytes);
    const int64_t nblk = ceil_div(n, kNB);
    float *bf = ar.take<float>(n);
    float *yz = ar.take<float>(2 * n);
    int *err = ar.take<int>(1);
    FLG_REQUIRE(bf && yz && err, "workspace too small for the low-precision solve");
    float *y = yz, *z = yz + n;
    // blocks per CTA: the chain crosses SMs once per q blocks; q grows only as far as the
    // CTAs' shared streams allow (one CTA per SM)
    int q = (int)std::max<int64_t>(kApplyQDefault, ceil_div(nblk, sm_count()));
    q = (int)std::min<int64_t>(q, nblk);
    FLG_REQUIRE(q <= kApplyQ, "low-precision solve: at most %lld unknowns", (long long)kApplyQ * sm_count() * kNB);
    const int G = (int)ceil_div(nblk, q);
    CUtensorMap mLU, mD;
    FLG_TRY(make_box_map_f32(&mLU, LU, n, n, ld, kNB, kNB));
    FLG_TRY(make_box_map_f32(&mD, dinv, 2 * nblk * kNB, kNB, kNB, kNB, kNB));
    d2f_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(b, bf, n);
    FLG_LAUNCH_CHECK();
    FLG_CUDA(cudaMemsetAsync(yz, 0xff, sizeof(float) * (size_t)(2 * n), st));  // the unset pattern
    FLG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    ApplyArgs aa{n, q, bf, y, z, err};
    void *args[] = {&mLU, &mD, &aa};
    FLG_TRY(lu_solve_lowp_prepare());
    prof_begin(FLG_SLOT_LU_SOLVE, st);
    FLG_CUDA(cudaLaunchCooperativeKernel((void *)lowp_apply_kernel, dim3(G), dim3(kApplyThreads), args, kApplySmem,
                                         st));
    count_launch();
    prof_end(FLG_SLOT_LU_SOLVE, st);
    f2d_kernel<<<(unsigned)ceil_div(n, 256), 256, 0, st>>>(z, x, n, err);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

}  // namespace flg

using namespace flg;

// ---- FP64 LU entry points --------------------------------------------------------------
static int panel_geometry(int64_t m, int &nblk, int &rpc) {
    const int sms = sm_count();
    nblk = (int)std::max<int64_t>(1, std::min<int64_t>(sms, ceil_div(m, 32)));
    rpc = (int)ceil_div(m, nblk);
    return rpc <= 384 ? FLG_OK : FLG_ERR_INVALID;
}

extern "C" size_t flg_lu_factor_f64_workspace(int64_t n) {
    CountingArena c;
    const int nblk = sm_count();
    c.take<GridBar>(1);
    c.take<unsigned long long>(2 * nblk);
    c.take<double>((size_t)2 * nblk * kRowBufLd);
    c.take<double>(2 * kPanel);
    (void)n;
    return c.bytes();
}

// Per host thread and device: the streams of the FP64 LU's look-ahead -- the next panel
// (highest priority) beside the trailing update, and the interchanges of the columns left of
// each panel (lowest priority), which nothing reads until the factorization ends.
struct F64Streams {
    int dev = -1;
    cudaStream_t panel = nullptr, left = nullptr;
    cudaEvent_t next_ready = nullptr, panel_done = nullptr, factored = nullptr, left_done = nullptr;
};
constexpr int kF64StreamDevices = 64;
static int f64_streams(F64Streams **out) {
    thread_local F64Streams per_dev[kF64StreamDevices];
    int dev = 0;
    FLG_CUDA(cudaGetDevice(&dev));
    FLG_REQUIRE(dev >= 0 && dev < kF64StreamDevices, "device ordinal %d out of range", dev);
    F64Streams &fs = per_dev[dev];
    if (fs.dev != dev) {
        int lo = 0, hi = 0;
        FLG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        FLG_CUDA(cudaStreamCreateWithPriority(&fs.panel, cudaStreamNonBlocking, hi));
        FLG_CUDA(cudaStreamCreateWithPriority(&fs.left, cudaStreamNonBlocking, lo));
        for (cudaEvent_t *e : {&fs.next_ready, &fs.panel_done, &fs.factored, &fs.left_done})
            FLG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        fs.dev = dev;
    }
    *out = &fs;
    return FLG_OK;
}

extern "C" int flg_lu_factor_f64(int64_t n, double *A, int64_t ld, int32_t *ipiv, int *info, void *work,
                                 size_t work_bytes, void *stream) {
    FLG_RANGE("flg_lu_factor_f64");
    FLG_REQUIRE(n >= 0 && ld >= n && info, "bad LU arguments");
    *info = 0;
    if (n == 0) return FLG_OK;
    FLG_REQUIRE(A && ipiv, "null pointer");
    int nblk0, rpc0;
    FLG_REQUIRE(panel_geometry(n, nblk0, rpc0) == FLG_OK, "FP64 dense LU supports n <= %d (use GMRES above)",
                sm_count() * 384);
    cudaStream_t st = as_stream(stream);
    Arena ar(work, work_bytes);
    const int maxblk = sm_count();
    GridBar *bar = ar.take<GridBar>(1);
    unsigned long long *word = ar.take<unsigned long long>(2 * maxblk);
    double *rowbuf = ar.take<double>((size_t)2 * maxblk * kRowBufLd);
    double *diagbuf = ar.take<double>(2 * kPanel);
    FLG_REQUIRE(diagbuf != nullptr, "workspace too small for LU (%zu bytes)", work_bytes);
    F64Streams *fs = nullptr;
    FLG_TRY(f64_streams(&fs));
    static bool attr_set = false;
    if (!attr_set) {
        FLG_CUDA(cudaFuncSetAttribute(panel_f64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      384 * kPanel * (int)sizeof(double)));
        for (const void *k : {(const void *)swap_trsm_kernel<true>, (const void *)swap_trsm_kernel<false>})
            FLG_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kPanel * kSwapThreads * (int)sizeof(double)));
        attr_set = true;
    }
    const size_t swap_smem = (size_t)kPanel * kSwapThreads * sizeof(double);
    FLG_CUDA(cudaMemsetAsync(bar, 0, sizeof(GridBar), st));
    // the panel of columns [k0, k0 + kb), rows k0.. on stream s
    auto panel = [&](int64_t k0, cudaStream_t s) -> int {
        const int kb = (int)std::min<int64_t>(kPanel, n - k0);
        const int64_t m = n - k0;
        int nblk, rpc;
        panel_geometry(m, nblk, rpc);
        int per_sm = 0;
        const size_t smem = (size_t)rpc * kb * sizeof(double);
        FLG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, panel_f64_kernel, 256, smem));
        FLG_REQUIRE(per_sm * sm_count() >= nblk, "panel grid (%d CTAs) cannot be co-resident", nblk);
        // both buffers of the published words to parity 1 (columns 0 and 1 expect parity 0)
        FLG_CUDA(cudaMemsetAsync(word, 0x80, 2 * (size_t)maxblk * sizeof(unsigned long long), s));
        PanelArgs pa{A, ld, n, k0, kb, rpc, ipiv, bar, word, rowbuf, diagbuf};
        void *args[] = {&pa};
        prof_begin(FLG_SLOT_LU_PANEL, s);
        FLG_CUDA(cudaLaunchCooperativeKernel((void *)panel_f64_kernel, dim3(nblk), dim3(256), args, smem, s));
        count_launch();
        prof_end(FLG_SLOT_LU_PANEL, s);
        return FLG_OK;
    };
    // Look-ahead: after each panel's trailing update has reached the next panel's 64 columns,
    // the next panel factors on the panel stream while the main stream updates the rest.
    // The interchanges of the columns left of each panel go to the left stream, in order.
    FLG_CUDA(cudaEventRecord(fs->factored, st));
    FLG_CUDA(cudaStreamWaitEvent(fs->left, fs->factored, 0));  // the left stream starts after prior work
    FLG_TRY(panel(0, st));
    bool ahead = false;  // the current panel ran ahead on the panel stream
    for (int64_t k0 = 0; k0 < n; k0 += kPanel) {
        const int kb = (int)std::min<int64_t>(kPanel, n - k0);
        if (ahead) FLG_CUDA(cudaStreamWaitEvent(st, fs->panel_done, 0));
        if (k0 > 0) {
            FLG_CUDA(cudaEventRecord(fs->factored, st));
            FLG_CUDA(cudaStreamWaitEvent(fs->left, fs->factored, 0));
            swap_trsm_kernel<false><<<(unsigned)ceil_div(k0, kSwapThreads), kSwapThreads, swap_smem, fs->left>>>(
                A, ld, ipiv, k0, kb, 0, k0);
            FLG_LAUNCH_CHECK();
        }
        const int64_t c0 = k0 + kb;
        ahead = false;
        if (c0 >= n) break;
        const int64_t nc = n - c0;
        swap_trsm_kernel<true><<<(unsigned)ceil_div(nc, kSwapThreads), kSwapThreads, swap_smem, st>>>(A, ld, ipiv, k0,
                                                                                                     kb, c0, n);
        FLG_LAUNCH_CHECK();
        prof_begin(FLG_SLOT_LU_UPDATE, st);
        const int64_t nn = std::min<int64_t>(kPanel, nc);  // the next panel's columns first
        dgemm_update_kernel<<<dim3((unsigned)ceil_div(nn, 64), (unsigned)ceil_div(nc, 64)), 256, 0, st>>>(
            A + c0 * ld + c0, A + c0 * ld + k0, A + k0 * ld + c0, ld, nc, nn, kb);
        FLG_LAUNCH_CHECK();
        if (nc > nn) {
            FLG_CUDA(cudaEventRecord(fs->next_ready, st));
            FLG_CUDA(cudaStreamWaitEvent(fs->panel, fs->next_ready, 0));
            FLG_TRY(panel(c0, fs->panel));
            FLG_CUDA(cudaEventRecord(fs->panel_done, fs->panel));
            ahead = true;
            dgemm_update_kernel<<<dim3((unsigned)ceil_div(nc - nn, 64), (unsigned)ceil_div(nc, 64)), 256, 0, st>>>(
                A + c0 * ld + c0 + nn, A + c0 * ld + k0, A + k0 * ld + c0 + nn, ld, nc, nc - nn, kb);
            FLG_LAUNCH_CHECK();
        }
        prof_end(FLG_SLOT_LU_UPDATE, st);
        if (!ahead) FLG_TRY(panel(c0, st));  // the last panel: nothing to overlap it with
    }
    FLG_CUDA(cudaEventRecord(fs->left_done, fs->left));
    FLG_CUDA(cudaStreamWaitEvent(st, fs->left_done, 0));
    GridBar hb;
    FLG_CUDA(cudaMemcpyAsync(&hb, bar, sizeof(GridBar), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    if (hb.err) {
        set_error("a bounded device wait timed out (LU panel exchange)");
        return FLG_ERR_TIMEOUT;
    }
    *info = hb.info;
    if (hb.info) {
        set_error("Matrix is singular (zero pivot at row %d)", hb.info - 1);
        return FLG_ERR_SINGULAR;
    }
    return FLG_OK;
}

extern "C" int flg_lu_solve_f64(int64_t n, int64_t nrhs, const double *LU, int64_t ld, const int32_t *ipiv, double *B,
                                int64_t ldb, void *stream) {
    FLG_RANGE("flg_lu_solve_f64");
    FLG_REQUIRE(n >= 0 && nrhs >= 0 && ld >= n && ldb >= nrhs, "bad LU solve arguments");
    if (n == 0 || nrhs == 0) return FLG_OK;
    cudaStream_t st = as_stream(stream);
    FLG_REQUIRE(nrhs <= 65535, "at most 65,535 right-hand sides per call");
    if (n <= kPivSmemMax) {
        static bool attr_set = false;
        if (!attr_set) {
            FLG_CUDA(cudaFuncSetAttribute(apply_pivots_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          kPivSmemMax * (int)sizeof(double)));
            attr_set = true;
        }
        apply_pivots_smem_kernel<<<(unsigned)nrhs, 256, n * sizeof(double), st>>>(B, ldb, ipiv, n);
    } else {
        apply_pivots_kernel<<<(unsigned)ceil_div(nrhs, 32), 32, 0, st>>>(B, ldb, nrhs, ipiv, n);
    }
    FLG_LAUNCH_CHECK();
    const int bsz = 64;
    for (int64_t b0 = 0; b0 < n; b0 += bsz) {
        const int bs = (int)std::min<int64_t>(bsz, n - b0);
        trsv_block_kernel<false><<<(unsigned)nrhs, 64, 0, st>>>(LU, ld, B, ldb, nrhs, b0, bs);
        FLG_LAUNCH_CHECK();
        if (b0 + bs < n) {
            const int64_t rows = n - b0 - bs;
            trsv_update_kernel<<<(unsigned)ceil_div(rows * nrhs * 32, 256), 256, 0, st>>>(LU, ld, B, ldb, nrhs, b0,
                                                                                         bs, b0 + bs, n);
            FLG_LAUNCH_CHECK();
        }
    }
    for (int64_t b0 = ((n - 1) / bsz) * bsz; b0 >= 0; b0 -= bsz) {
        const int bs = (int)std::min<int64_t>(bsz, n - b0);
        trsv_block_kernel<true><<<(unsigned)nrhs, 64, 0, st>>>(LU, ld, B, ldb, nrhs, b0, bs);
        FLG_LAUNCH_CHECK();
        if (b0 > 0) {
            trsv_update_kernel<<<(unsigned)ceil_div(b0 * nrhs * 32, 256), 256, 0, st>>>(LU, ld, B, ldb, nrhs, b0, bs,
                                                                                       0, b0);
            FLG_LAUNCH_CHECK();
        }
    }
    return FLG_OK;
}

// ---- low-precision LU entry points ----------------------------------------------------
// Per host thread and device: the stream that runs the next diagonal block while the
// trailing update finishes (highest priority), and the events of that fork and join.
// Created on first use; an LU captured in a graph makes one eager pass first.
// One set per device ordinal, so a thread that moves between GPUs keeps (and reuses) each
// device's stream and events instead of creating new ones on every switch.
struct SideStream {
    int dev = -1;
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, tail = nullptr, lfork = nullptr, ljoin = nullptr;
};
constexpr int kSideStreamDevices = 64;
static int side_stream(SideStream **out) {
    thread_local SideStream per_dev[kSideStreamDevices];
    int dev = 0;
    FLG_CUDA(cudaGetDevice(&dev));
    FLG_REQUIRE(dev >= 0 && dev < kSideStreamDevices, "device ordinal %d out of range", dev);
    SideStream &ss = per_dev[dev];
    if (ss.dev != dev) {
        int lo = 0, hi = 0;
        FLG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        FLG_CUDA(cudaStreamCreateWithPriority(&ss.s, cudaStreamNonBlocking, hi));
        FLG_CUDA(cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming));
        FLG_CUDA(cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming));
        FLG_CUDA(cudaEventCreateWithFlags(&ss.tail, cudaEventDisableTiming));
        FLG_CUDA(cudaEventCreateWithFlags(&ss.lfork, cudaEventDisableTiming));
        FLG_CUDA(cudaEventCreateWithFlags(&ss.ljoin, cudaEventDisableTiming));
        ss.dev = dev;
    }
    *out = &ss;
    return FLG_OK;
}

extern "C" int64_t flg_lu_lowp_dinv_elems(int64_t n) { return 2 * ceil_div(std::max<int64_t>(n, 1), kNB) * kNB * kNB; }

// Tensor-core modes defer most of the trailing update: blocks are grouped into
// outer panels of W columns [K0, E), W = outer_width(n).  Inner step k0 (diagonal block,
// panels) updates only the L-shaped part of the Schur complement that the next
// inner steps read -- rows > k0 x columns (k0, E), and rows (k0, E) x columns
// >= E -- with rank-128 updates; the rest, rows and columns >= E, receives one
// rank-(E - K0) update per outer panel, which moves the trailing matrix through
// HBM W / 128 times less often.  The K-major copy of U (UtB: one row of W
// per column >= K0) feeds both.  A wider W halves the trailing traffic again but
// lengthens the chain of inner steps that nothing overlaps; measured on the
// tensor-core modes (TF32 / BF16, factor + refinement): 1,024 columns is 6-9%
// faster from n = 12,288 up and 2% slower at n = 4,608, so 512 below n = 8,192.
static int64_t outer_width(int64_t n) { return (n >= 8192 ? 8 : 4) * (int64_t)kNB; }

// scratch of nbat systems, system z's at + z * (kNB n, n kNB, n W) floats; BF16 mode: the
// BF16 copies of the outer panel's L columns and of UtB (n W each per system) in PB
template <class Ar>
static void lowp_carve(Ar &ar, int64_t n, int nbat, int mode, float **U12, float **L21, float **UtB, char **tcw,
                       size_t *tcb, __nv_bfloat16 **PB) {
    *U12 = ar.template take<float>((size_t)nbat * kNB * n);
    *L21 = ar.template take<float>((size_t)nbat * n * kNB);
    const int64_t W = outer_width(n);
    *UtB = ar.template take<float>((size_t)nbat * n * W);
    // the panel products run in TF32 (no operand workspace); the BF16 updates read PB
    *tcb = (mode == FLG_LU_FP32) ? 0 : tc_update_bytes(n, n, W, FLG_LU_TF32, nbat);
    *tcw = ar.template take<char>(*tcb);
    *PB = mode == FLG_LU_BF16 ? ar.template take<__nv_bfloat16>((size_t)2 * nbat * n * W) : nullptr;
}

// precision part of an LU mode (the tile bits masked off)
static int lu_prec(int mode) { return mode & ~(FLG_LU_TILE_N128 | FLG_LU_TILE_N256); }

extern "C" size_t flg_lu_factor_lowp_workspace(int64_t n, int mode) {
    mode = lu_prec(mode);
    CountingArena c;
    float *a, *b, *d;
    char *w;
    size_t t;
    __nv_bfloat16 *pb;
    lowp_carve(c, n, 1, mode, &a, &b, &d, &w, &t, &pb);
    return c.bytes() + 256;  // + the flags of flg_lu_factor_lowp, at the end
}

extern "C" size_t flg_lu_factor_lowp_batched_workspace(int64_t n, int nbat, int mode) {
    mode = lu_prec(mode);
    CountingArena c;
    float *a, *b, *d;
    char *w;
    size_t t;
    __nv_bfloat16 *pb;
    lowp_carve(c, n, std::max(nbat, 1), mode, &a, &b, &d, &w, &t, &pb);
    return c.bytes();
}

// The low-precision LU of nbat systems of order n in one sequence of launches: system z at
// A + z sA (row stride ld), its block inverses at dinv + z flg_lu_lowp_dinv_elems(n), its
// flags at flags + 2 z.  Every kernel of a step covers all systems (one CTA per system for
// the diagonal blocks; the tensor-core updates walk the tiles of all systems).
static int lowp_factor(int64_t n, int nbat, float *A, int64_t ld, int64_t sA, int mode, float *dinv, int *flags,
                       void *work, size_t work_bytes, cudaStream_t st) {
    FLG_REQUIRE(n >= 0 && ld >= n && flags && nbat >= 1, "bad LU arguments");
    const int tbits = mode & (FLG_LU_TILE_N128 | FLG_LU_TILE_N256);
    FLG_REQUIRE(tbits != (FLG_LU_TILE_N128 | FLG_LU_TILE_N256), "two tile widths in LU mode %d", mode);
    const int tile = tbits == FLG_LU_TILE_N128 ? 128 : tbits == FLG_LU_TILE_N256 ? 256 : 0;
    mode = lu_prec(mode);
    FLG_REQUIRE(mode == FLG_LU_TF32 || mode == FLG_LU_BF16 || (mode == FLG_LU_FP32 && tile == 0), "unknown LU mode %d",
                mode | tbits);
    FLG_REQUIRE(nbat == 1 || mode != FLG_LU_FP32, "batched LU needs a tensor-core mode (TF32 or BF16)");
    FLG_REQUIRE(nbat == 1 || (sA >= n * ld && sA % 4 == 0), "bad system stride");
    FLG_REQUIRE(ld % 4 == 0, "ld must be a multiple of 4 (16-byte rows)");
    FLG_CUDA(cudaMemsetAsync(flags, 0, 2 * sizeof(int) * nbat, st));
    if (n == 0) return FLG_OK;
    FLG_REQUIRE(A && dinv, "null pointer");
    Arena ar(work, work_bytes);
    float *U12, *L21, *UtB;
    char *tcw;
    size_t tcb;
    __nv_bfloat16 *PB;
    lowp_carve(ar, n, nbat, mode, &U12, &L21, &UtB, &tcw, &tcb, &PB);
    FLG_REQUIRE(U12 && L21 && UtB && (tcb == 0 || tcw) && (mode != FLG_LU_BF16 || PB),
                "workspace too small for LU (%zu bytes)", work_bytes);
    // the tensor-core panels use the partial-block scratch: U12 for A12^T, L21 for Uinv^T
    float *T12 = U12, *UinvT = L21;
    int *dinfo = flags;  // [0] first bad pivot, [1] tensor-core wait timed out
    const int64_t W = outer_width(n);  // outer panel width
    // per-system strides: the matrix, the block inverses, A12^T / Uinv^T scratch, U's K-major copy
    const int64_t sD = flg_lu_lowp_dinv_elems(n), sT = (int64_t)kNB * n, sUt = n * W;
    const TcBatch bA{nbat, sA, sA, sUt}, bU{nbat, sUt, sT, sD}, bL{nbat, sA, sA, sT};
    // BF16 mode: each step's finished L and U panels are rounded once into LB (row r, column
    // c - K0 of the outer panel at LB + r W + c - K0) and UB (laid out as UtB), and every
    // trailing update of the outer panel reads them
    __nv_bfloat16 *LB = PB, *UB = PB ? PB + (size_t)nbat * n * W : nullptr;
    const TcBatch bB{nbat, sA, n * W, n * W};
    int64_t K0 = 0;  // first column of the current outer panel
    // C -= Lp Up^T (Lp inside A at columns [K0, E), Up inside UtB) over m x nc, depth K
    auto upd = [&](float *C, const float *Lp, const float *Up, int64_t m, int64_t nc, int64_t K, int ctas) -> int {
        if (mode == FLG_LU_BF16) {
            const int64_t off = Lp - A, r = off / ld, c = off % ld;
            return tc_update_bf16(C, ld, LB + r * W + (c - K0), W, UB + (Up - UtB), W, m, nc, K, tcw, tcb, st,
                                  dinfo + 1, tile, ctas, bB);
        }
        return tc_update(C, ld, Lp, ld, Up, W, m, nc, K, mode, tcw, tcb, st, dinfo + 1, false, tile, ctas, bA);
    };
    const size_t dsmem = kDiagSmem;
    static bool attr_set = false;  // set once, so a later call can be captured in a graph
    if (!attr_set) {
        FLG_CUDA(cudaFuncSetAttribute(diag_lowp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsmem));
        attr_set = true;
    }
    const bool tc = mode != FLG_LU_FP32;
    const int64_t nblk = ceil_div(n, kNB);
    float *Linv = dinv, *Uinv = dinv + nblk * kNB * kNB;
    SideStream *side = nullptr;
    if (tc) FLG_TRY(side_stream(&side));
    // the persistent updates that run beside the look-ahead diagonal blocks leave them an SM each
    const int cap = std::max(1, sm_count() - nbat);
    auto diag = [&](int64_t d0, cudaStream_t s) {
        const int64_t kd = d0 / kNB;
        const int nbd = (int)std::min<int64_t>(kNB, n - d0);
        const bool tcp = tc && nbd == kNB && n - (d0 + nbd) > 0;  // tensor-core panels follow
        prof_begin(FLG_SLOT_LU_DIAG, s);
        diag_lowp_kernel<<<nbat, 512, dsmem, s>>>(A, ld, d0, nbd, Linv + kd * kNB * kNB, Uinv + kd * kNB * kNB,
                                                  tcp ? UinvT : nullptr, dinfo, sA, sD, sT);
        prof_end(FLG_SLOT_LU_DIAG, s);
    };
    // Look-ahead: once the 128 x 128 block at d0 has its last update (launched on st), the
    // diagonal kernel of that block runs on the side stream while st goes on with the rest of
    // the trailing update; the next panels wait for it.  Only for a full block with a
    // trailing part (the block's own panels then run on the tensor cores).
    bool pending = false, side_busy = false;
    const dim3 tb(32, 8);
    // Ut of an inner step back into the row block A12 (U12 row-major, read only by the solves):
    // off the critical path, after the join on the side stream.  The next panels write other
    // K slots of UtB and another row block; the next outer panel rewrites UtB only after a
    // later diagonal kernel on the side stream, so every deferred transpose has run by then.
    struct Deferred {
        const float *Ut = nullptr;
        float *A12 = nullptr;
        int64_t nr = 0;
    };
    auto look_ahead = [&](int64_t d0, Deferred t) -> int {
        FLG_CUDA(cudaEventRecord(side->fork, st));
        FLG_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
        diag(d0, side->s);
        FLG_LAUNCH_CHECK();
        FLG_CUDA(cudaEventRecord(side->join, side->s));
        if (t.Ut) {
            transpose_f32_kernel<<<dim3(kNB / 32, (unsigned)ceil_div(t.nr, 32), nbat), tb, 0, side->s>>>(
                t.Ut, W, t.A12, ld, t.nr, kNB, sUt, sA);
            FLG_LAUNCH_CHECK();
            side_busy = true;
        }
        pending = true;
        return FLG_OK;
    };
    for (K0 = 0; K0 < n; K0 += W) {
        const int64_t E = std::min<int64_t>(n, K0 + W);
        for (int64_t k0 = K0; k0 < E; k0 += kNB) {
            const int64_t k = k0 / kNB;
            const int nb = (int)std::min<int64_t>(kNB, n - k0);
            const bool tcp = tc && nb == kNB && n - (k0 + nb) > 0;  // tensor-core panels
            if (pending) {  // this block's diagonal kernel ran ahead on the side stream
                FLG_CUDA(cudaStreamWaitEvent(st, side->join, 0));
                pending = false;
            } else {
                diag(k0, st);
                FLG_LAUNCH_CHECK();
            }
            const int64_t c0 = k0 + nb, nr = n - c0;
            if (nr <= 0) continue;
            prof_begin(FLG_SLOT_LU_PANEL, st);
            // (nb < kNB only for the last block, which has no trailing part)
            float *A12 = A + k0 * ld + c0, *A21 = A + c0 * ld + k0, *A22 = A + c0 * ld + c0;
            float *Ut = UtB + (c0 - K0) * W + (k0 - K0);  // row: column - K0; K offset: k0 - K0
            // an inner step whose next diagonal block runs ahead defers its transpose-back
            const bool defer_t = tcp && E > c0 && n - c0 > kNB;
            if (tcp) {
                // panels on the tensor cores (TF32 in both tensor-core modes):
                //   Ut = A12^T Linv^T (the K-major copy the updates read), then A12 = Ut^T;
                //   L21 = A21 Uinv, in place (each tile's rows are read in full before they are stored),
                //   on the side stream beside the U panel (TF32 store mode touches no shared
                //   workspace); the updates below join it, and the next diagonal kernel, which
                //   rewrites Uinv^T, follows it on the side stream
                FLG_CUDA(cudaEventRecord(side->lfork, st));
                FLG_CUDA(cudaStreamWaitEvent(side->s, side->lfork, 0));
                FLG_TRY(tc_update(A21, ld, A21, ld, UinvT, kNB, nr, kNB, kNB, FLG_LU_TF32, tcw, tcb, side->s,
                                  dinfo + 1, true, 0, 0, bL));
                FLG_CUDA(cudaEventRecord(side->ljoin, side->s));
                transpose_f32_kernel<<<dim3((unsigned)ceil_div(nr, 32), kNB / 32, nbat), tb, 0, st>>>(
                    A12, ld, T12, kNB, kNB, nr, sA, sT);
                FLG_LAUNCH_CHECK();
                FLG_TRY(tc_update(Ut, W, T12, kNB, Linv + k * kNB * kNB, kNB, nr, kNB, kNB, FLG_LU_TF32, tcw,
                                  tcb, st, dinfo + 1, true, 0, 0, bU));
                if (!defer_t) {
                    transpose_f32_kernel<<<dim3(kNB / 32, (unsigned)ceil_div(nr, 32), nbat), tb, 0, st>>>(
                        Ut, W, A12, ld, nr, kNB, sUt, sA);
                    FLG_LAUNCH_CHECK();
                }
                FLG_CUDA(cudaStreamWaitEvent(st, side->ljoin, 0));
                if (mode == FLG_LU_BF16) {  // both panels of this step, rounded once for every update
                    panel_bf16_kernel<<<dim3((unsigned)ceil_div(nr * 32, 256), 2, nbat), 256, 0, st>>>(
                        A21, ld, Ut, W, LB + c0 * W + (k0 - K0), UB + (Ut - UtB), W, nr, sA, sUt, n * W);
                    FLG_LAUNCH_CHECK();
                }
            } else if (nb == kNB) {
                // U12 = Linv A12 (+ its K-major copy), L21 = A21 Uinv: one launch, in place
                const int ntu = (int)ceil_div(nr, 32), ntl = (int)ceil_div(nr, 32);
                lowp_panel_kernel<<<ntu + ntl, 256, 0, st>>>(A, ld, k0, nr, Linv + k * kNB * kNB, Uinv + k * kNB * kNB,
                                                             Ut, W, ntu);
                FLG_LAUNCH_CHECK();
            } else {
                FLG_TRY(sgemm(st, nb, nr, nb, 1.0f, Linv + k * kNB * kNB, kNB, A12, ld, 0.0f, U12, nr));
                FLG_TRY(copy2d(st, U12, nr, A12, ld, nb, nr));
                FLG_TRY(sgemm(st, nr, nb, nb, 1.0f, A21, ld, Uinv + k * kNB * kNB, kNB, 0.0f, L21, kNB));
                FLG_TRY(copy2d(st, L21, kNB, A21, ld, nr, nb));
            }
            prof_end(FLG_SLOT_LU_PANEL, st);
            prof_begin(FLG_SLOT_LU_UPDATE, st);
            if (!tc || nb < kNB) {
                FLG_TRY(sgemm(st, nr, nr, nb, -1.0f, A21, ld, A12, ld, 1.0f, A22, ld));
            } else if (E > c0) {
                if (n - c0 > kNB) {
                    // the next diagonal block first, then it factors beside the rest:
                    // rows > c0 + 128 x its columns, rows > k0 x columns (c0 + 128, E)
                    FLG_TRY(upd(A22, A21, Ut, kNB, kNB, kNB, 0));
                    FLG_TRY(look_ahead(c0, Deferred{Ut, A12, nr}));
                    FLG_TRY(upd(A22 + kNB * ld, A21 + kNB * ld, Ut, nr - kNB, kNB, kNB, cap));
                    if (E > c0 + kNB) FLG_TRY(upd(A22 + kNB, A21, Ut + kNB * W, nr, E - c0 - kNB, kNB, cap));
                } else {
                    // rows > k0 x columns (k0, E)
                    FLG_TRY(upd(A22, A21, Ut, nr, E - c0, kNB, 0));
                }
                // rows (k0, E) x columns >= E
                if (n > E) FLG_TRY(upd(A + c0 * ld + E, A21, Ut + (E - c0) * W, E - c0, n - E, kNB, pending ? cap : 0));
            }
            prof_end(FLG_SLOT_LU_UPDATE, st);
        }
        if (tc && n > E) {  // the deferred rank-(E - K0) update of rows and columns >= E (E - K0 = W here)
            prof_begin(FLG_SLOT_LU_UPDATE, st);
            float *C = A + E * ld + E, *Lp = A + E * ld + K0, *Up = UtB + (E - K0) * W;
            if (n - E > kNB) {
                // the next outer panel's first diagonal block first, then it factors beside the rest
                FLG_TRY(upd(C, Lp, Up, kNB, kNB, E - K0, 0));
                FLG_TRY(look_ahead(E, Deferred{}));
                FLG_TRY(upd(C + kNB * ld, Lp + kNB * ld, Up, n - E - kNB, kNB, E - K0, cap));
                FLG_TRY(upd(C + kNB, Lp, Up + kNB * W, n - E, n - E - kNB, E - K0, cap));
            } else {
                FLG_TRY(upd(C, Lp, Up, n - E, n - E, E - K0, 0));
            }
            prof_end(FLG_SLOT_LU_UPDATE, st);
        }
    }
    if (pending) FLG_CUDA(cudaStreamWaitEvent(st, side->join, 0));  // (every look-ahead is joined above)
    if (side_busy) {  // the deferred transposes
        FLG_CUDA(cudaEventRecord(side->tail, side->s));
        FLG_CUDA(cudaStreamWaitEvent(st, side->tail, 0));
    }
    return FLG_OK;
}

extern "C" int flg_lu_factor_lowp_async(int64_t n, float *A, int64_t ld, int mode, float *dinv, int *flags, void *work,
                                        size_t work_bytes, void *stream) {
    FLG_RANGE("flg_lu_factor_lowp_async");
    return lowp_factor(n, 1, A, ld, 0, mode, dinv, flags, work, work_bytes, as_stream(stream));
}

extern "C" int flg_lu_factor_lowp_batched_async(int64_t n, int nbat, float *A, int64_t ld, int64_t stride_a, int mode,
                                                float *dinv, int *flags, void *work, size_t work_bytes,
                                                void *stream) {
    FLG_RANGE("flg_lu_factor_lowp_batched_async");
    FLG_REQUIRE(nbat >= 1 && nbat <= 64, "batch of %d systems (1 .. 64)", nbat);
    return lowp_factor(n, nbat, A, ld, stride_a, mode, dinv, flags, work, work_bytes, as_stream(stream));
}

extern "C" int flg_lu_factor_lowp(int64_t n, float *A, int64_t ld, int mode, float *dinv, int *info, void *work,
                                  size_t work_bytes, void *stream) {
    FLG_RANGE("flg_lu_factor_lowp");
    FLG_REQUIRE(info, "null info");
    *info = 0;
    FLG_REQUIRE(n >= 0 && ld >= n, "bad LU arguments");
    if (n == 0) return FLG_OK;
    // the two device flags live at the end of the workspace
    const size_t need = flg_lu_factor_lowp_workspace(n, mode);
    FLG_REQUIRE(work && work_bytes >= need, "workspace too small for LU (%zu bytes, %zu needed)", work_bytes, need);
    int *flags = (int *)((char *)work + ((need - 64) & ~size_t(15)));
    cudaStream_t st = as_stream(stream);
    FLG_TRY(flg_lu_factor_lowp_async(n, A, ld, mode, dinv, flags, work, need - 128, stream));
    int hflags[2] = {0, 0};
    FLG_CUDA(cudaMemcpyAsync(hflags, flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    if (hflags[1]) {
        set_error("a bounded device wait timed out (tensor-core update or diagonal block)");
        return FLG_ERR_TIMEOUT;
    }
    *info = hflags[0];
    if (hflags[0]) {
        set_error("zero or non-finite pivot at row %d in the low-precision LU", hflags[0] - 1);
        return FLG_ERR_SINGULAR;
    }
    return FLG_OK;
}

extern "C" size_t flg_lu_solve_lowp_workspace(int64_t n) { return lu_solve_lowp_bytes(n); }

extern "C" int flg_lu_solve_lowp(int64_t n, const float *LU, int64_t ld, const float *dinv, const double *b, double *x,
                                 void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_lu_solve_lowp");
    FLG_REQUIRE(n >= 0 && ld >= n, "bad solve arguments");
    if (n == 0) return FLG_OK;
    return lu_solve_lowp_apply(n, LU, ld, dinv, b, x, work, work_bytes, as_stream(stream));
}
