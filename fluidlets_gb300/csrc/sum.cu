// sum.cu -- kernel sums u_i = sum_j G(x_i, y_j; eps_j) f_j / mu.
//
// Replaces fluidlets.evaluate (core/matvec.py:24-49) and its Numba loop
// _apply (core/matvec.py:10-21).  Two precisions:
//
//  FLG_PREC_FP64  sum_f64_kernel: one target per thread, sources staged in
//                 shared memory in tiles of 128, FP64 arithmetic throughout.
//  FLG_PREC_MIXED far_f32_kernel: TPT targets per thread, 256-source tiles of
//                 packed FP32 sources (float4 x,y,z,eps^2 | f0,f1,f2,thr) in
//                 cell order, register-prefetched; pairs with r < 4 eps_j are
//                 masked out -- except in tiles whose bounding box lies
//                 beyond every threshold from the box of the CTA's targets
//                 (targets taken in cell order too, so that both boxes are
//                 small), which run without the mask; FP32 accumulation
//                 within a tile, FP64 across tiles.
//                 near_f64_kernel: a uniform cell list (cell >= 4.2 max eps)
//                 finds the masked pairs, which are summed in FP64 with the
//                 same predicate, then the partial sums are combined.
//
// Both paths split the sources over gridDim.y so that small target counts
// still fill the 152 SMs; the per-split partial sums go to workspace and are
// combined in a fixed order (bitwise deterministic results).
#include <algorithm>
#include <mutex>

#include "flg_common.cuh"
#include "pair_math.cuh"
#include "sum_plan.cuh"

namespace flg {

constexpr int kF64Threads = 128;
constexpr int kF64Tile = 128;
constexpr int kF32Threads = 256;
constexpr int kF32Tile = 256;
constexpr int kMaxCells = 1 << 20;
constexpr int kBoundBlocks = 256;
constexpr int kScanBlock = 1024;  // elements per scan block (one per thread)
constexpr int64_t kSortTargetsMin = 32768;  // mixed sums bucket larger target sets by cell

__host__ __device__ inline int out_width(int nf, bool ck) { return (nf == 2 || ck) ? 6 : 3; }

struct SumArgs {
    const double *tg;
    int64_t M;
    const double *src;
    const double *eps;
    const double *f;
    int64_t N;
    int64_t split_len;
    double alpha_re, alpha_im;
    double *partial;  // [S][M][OUTW]
};

// Strength of source j as 3*NF doubles: [f0, f1, f2] (real), or
// [re f0, re f1, re f2, im f0, im f1, im f2] from interleaved complex128.
template <int NF>
__device__ __forceinline__ void load_strength(const double *f, int64_t j, double *out) {
    if constexpr (NF == 1) {
#pragma unroll
        for (int c = 0; c < 3; c++) out[c] = f[3 * j + c];
    } else {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            out[c] = f[6 * j + 2 * c];
            out[3 + c] = f[6 * j + 2 * c + 1];
        }
    }
}

// ---------------------------------------------------------------------------
// per-pair accumulation shared by the FP64 kernels (plain sum and near field)
// ---------------------------------------------------------------------------
template <int KIND, int NF, bool CK>
__device__ __forceinline__ void pair_f64(double tx, double ty, double tz, double tz2, double sx, double sy,
                                         double sz, double e2, const double *fj, double are, double aim,
                                         double *u) {
    if constexpr (KIND == FLG_WALL) {
        WallGeo<double> g = wall_geo<double, false>(tx, ty, tz, tz2, sx, sy, sz, e2, 0.0);
        wall_apply(g, fj[0], fj[1], fj[2], u);
        if constexpr (NF == 2) wall_apply(g, fj[3], fj[4], fj[5], u + 3);
    } else {
        double d0 = tx - sx, d1 = ty - sy, d2 = tz - sz;
        double Q = fma(d2, d2, fma(d1, d1, fma(d0, d0, e2)));
        double s = rsq(Q);
        if constexpr (CK) {
            cpx<double> A, B;
            brink_AB_c<double>(s, Q, e2, are, aim, A, B);
            if constexpr (NF == 1) {
                radial_apply(A.re, B.re, d0, d1, d2, fj[0], fj[1], fj[2], u);
                radial_apply(A.im, B.im, d0, d1, d2, fj[0], fj[1], fj[2], u + 3);
            } else {
                // (A_re + i A_im)(f_re + i f_im): re += A_re f_re - A_im f_im, im += A_re f_im + A_im f_re
                radial_apply(A.re, B.re, d0, d1, d2, fj[0], fj[1], fj[2], u);
                radial_apply(-A.im, -B.im, d0, d1, d2, fj[3], fj[4], fj[5], u);
                radial_apply(A.re, B.re, d0, d1, d2, fj[3], fj[4], fj[5], u + 3);
                radial_apply(A.im, B.im, d0, d1, d2, fj[0], fj[1], fj[2], u + 3);
            }
        } else {
            double A, B;
            if constexpr (KIND == FLG_STOKESLET) stokeslet_AB(s, e2, A, B);
            else brink_AB<double>(s, Q, e2, are, A, B);
            radial_apply(A, B, d0, d1, d2, fj[0], fj[1], fj[2], u);
            if constexpr (NF == 2) radial_apply(A, B, d0, d1, d2, fj[3], fj[4], fj[5], u + 3);
        }
    }
}

// ---------------------------------------------------------------------------
// FP64 plain sum
// ---------------------------------------------------------------------------
template <int KIND, int NF, bool CK>
__global__ void __launch_bounds__(kF64Threads) sum_f64_kernel(SumArgs a) {
    constexpr int OUTW = (NF == 2 || CK) ? 6 : 3;
    __shared__ double s_p[kF64Tile][4];
    __shared__ double s_f[kF64Tile][3 * NF];
    const int64_t i = (int64_t)blockIdx.x * kF64Threads + threadIdx.x;
    const int64_t ii = i < a.M ? i : a.M - 1;
    const double tx = a.tg[3 * ii], ty = a.tg[3 * ii + 1], tz = a.tg[3 * ii + 2];
    const double tz2 = 2.0 * tz;
    double u[OUTW];
#pragma unroll
    for (int c = 0; c < OUTW; c++) u[c] = 0.0;
    const int64_t j0 = (int64_t)blockIdx.y * a.split_len;
    const int64_t j1 = min(a.N, j0 + a.split_len);
    for (int64_t jt = j0; jt < j1; jt += kF64Tile) {
        const int cnt = (int)(j1 - jt < kF64Tile ? j1 - jt : kF64Tile);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += kF64Threads) {
            const int64_t j = jt + k;
            s_p[k][0] = a.src[3 * j];
            s_p[k][1] = a.src[3 * j + 1];
            s_p[k][2] = a.src[3 * j + 2];
            const double e = a.eps[j];
            s_p[k][3] = e * e;
            load_strength<NF>(a.f, j, s_f[k]);
        }
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < cnt; k++) {
            pair_f64<KIND, NF, CK>(tx, ty, tz, tz2, s_p[k][0], s_p[k][1], s_p[k][2], s_p[k][3], s_f[k], a.alpha_re,
                                   a.alpha_im, u);
        }
    }
    if (i < a.M) {
        double *p = a.partial + ((int64_t)blockIdx.y * a.M + i) * OUTW;
#pragma unroll
        for (int c = 0; c < OUTW; c++) p[c] = u[c];
    }
}

// ---------------------------------------------------------------------------
// finalize: out = (sum_s partial[s] + near) * scale / mu
// ---------------------------------------------------------------------------
struct FinalArgs {
    const double *partial;
    int S;
    int64_t M;
    int outw;
    const double *near;  // [M][outw] or null
    double scale;
    int out_complex;
    int mu_complex;
    double mu_re;             // real mu
    int mu_branch;            // Smith's complex division
    double mu_rat, mu_scl;
    double *out;
};

__device__ __forceinline__ void final_store(const FinalArgs &a, int64_t i, const double *u) {
    if (!a.out_complex) {
#pragma unroll
        for (int c = 0; c < 3; c++) a.out[3 * i + c] = (u[c] * a.scale) / a.mu_re;
        return;
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double xr = u[c] * a.scale;
        double xi = a.outw == 6 ? u[3 + c] * a.scale : 0.0;
        double yr, yi;
        if (!a.mu_complex) {
            yr = xr / a.mu_re;
            yi = xi / a.mu_re;
        } else if (a.mu_branch == 0) {  // |mu_re| >= |mu_im|
            yr = (xr + xi * a.mu_rat) * a.mu_scl;
            yi = (xi - xr * a.mu_rat) * a.mu_scl;
        } else {
            yr = (xr * a.mu_rat + xi) * a.mu_scl;
            yi = (xi * a.mu_rat - xr) * a.mu_scl;
        }
        a.out[6 * i + 2 * c] = yr;
        a.out[6 * i + 2 * c + 1] = yi;
    }
}

__global__ void finalize_kernel(FinalArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.M) return;
    double u[6] = {0, 0, 0, 0, 0, 0};
    for (int s = 0; s < a.S; s++) {
        const double *p = a.partial + ((int64_t)s * a.M + i) * a.outw;
        for (int c = 0; c < a.outw; c++) u[c] += p[c];
    }
    if (a.near)
        for (int c = 0; c < a.outw; c++) u[c] += a.near[i * a.outw + c];
    final_store(a, i, u);
}

// ---------------------------------------------------------------------------
// FP32 far field
// ---------------------------------------------------------------------------
struct FarArgs {
    const double *tg;
    int64_t M;
    const int *tperm;      // processing position -> target index (null: identity)
    const float4 *packed;  // [N][NQ]
    const float4 *tile_box;  // [N / 256][2]
    int64_t N;
    int64_t split_len;
    float alpha_re, alpha_im;
    double *partial;  // [S][M][OUTW], by processing position
};

template <int KIND, int NF, bool CK, bool MASK = true>
__device__ __forceinline__ void pair_f32_far(float tx, float ty, float tz, float tz2, const float4 &p,
                                             const float4 &q, const float4 &r, float are, float aim, float *u) {
    // p = {x, y, z, e2}; q = {f0, f1, f2, thr}; r = {f0i, f1i, f2i, 0}
    if constexpr (KIND == FLG_WALL) {
        // strengths arrive scaled by the source height; the caller applies 2 t per tile
        (void)tz2;
        const WallFar g = wall_far_geo<MASK>(tx, ty, tz, p.x, p.y, p.z, p.w, q.w);
        wall_far_acc(g, q.x, q.y, q.z, u);
        if constexpr (NF == 2) wall_far_acc(g, r.x, r.y, r.z, u + 3);
    } else {
        float d0 = sub_rn(tx, p.x), d1 = sub_rn(ty, p.y), d2 = sub_rn(tz, p.z);
        float Q = free_Q_f32(d0, d1, d2, p.w);
        float s = rsq(Q);
        if (MASK) s = (Q < q.w) ? 0.0f : s;  // near pair: summed in FP64 by near_f64_kernel
        if constexpr (CK) {
            cpx<float> A, B;
            brink_AB_c<float>(s, Q, p.w, are, aim, A, B);
            if constexpr (NF == 1) {
                radial_apply(A.re, B.re, d0, d1, d2, q.x, q.y, q.z, u);
                radial_apply(A.im, B.im, d0, d1, d2, q.x, q.y, q.z, u + 3);
            } else {
                radial_apply(A.re, B.re, d0, d1, d2, q.x, q.y, q.z, u);
                radial_apply(-A.im, -B.im, d0, d1, d2, r.x, r.y, r.z, u);
                radial_apply(A.re, B.re, d0, d1, d2, r.x, r.y, r.z, u + 3);
                radial_apply(A.im, B.im, d0, d1, d2, q.x, q.y, q.z, u + 3);
            }
        } else {
            float A, B;
            if constexpr (KIND == FLG_STOKESLET) stokeslet_AB(s, p.w, A, B);
            else brink_AB<float>(s, Q, p.w, are, A, B);
            radial_apply(A, B, d0, d1, d2, q.x, q.y, q.z, u);
            if constexpr (NF == 2) radial_apply(A, B, d0, d1, d2, r.x, r.y, r.z, u + 3);
        }
    }
}

// Code generation of the far-field kernel, measured on GB300 (all kernel kinds as fast or
// faster than without them): at least 3 CTAs per SM (80 registers at most), and the
// unmasked loop unrolled 4 deep.  0 CTAs leaves the register count to the compiler.
#ifndef FLG_FAR_MINB
#define FLG_FAR_MINB 3
#endif
#if FLG_FAR_MINB > 0
#define FLG_FAR_BOUNDS __launch_bounds__(kF32Threads, FLG_FAR_MINB)
#else
#define FLG_FAR_BOUNDS __launch_bounds__(kF32Threads)
#endif
#ifndef FLG_FAR_UNROLL
#define FLG_FAR_UNROLL 4
#endif
constexpr int kFarUnroll = FLG_FAR_UNROLL;
template <int KIND, int NF, bool CK, int TPT>
__global__ void FLG_FAR_BOUNDS far_f32_kernel(FarArgs a) {
    constexpr int NQ = 1 + NF;
    constexpr int OUTW = (NF == 2 || CK) ? 6 : 3;
    // the wall kernel's targets run the far loop two per register pair, in packed FP32x2
    // arithmetic, from a copy of the tile with every source value duplicated into both halves
    constexpr bool PACK = KIND == FLG_WALL && NF == 1 && !CK && TPT % 2 == 0;
    __shared__ float4 s_src[kF32Tile * NQ];
    __shared__ ulonglong2 s_dup[PACK ? kF32Tile * 4 : 1];
    __shared__ float s_box[kF32Threads / 32][6];
    const int64_t base = (int64_t)blockIdx.x * (kF32Threads * TPT) + threadIdx.x;
    float tx[TPT], ty[TPT], tz[TPT], tz2[TPT];
    float bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
#pragma unroll
    for (int t = 0; t < TPT; t++) {
        int64_t k = base + (int64_t)t * kF32Threads;
        k = k < a.M ? k : a.M - 1;
        const int64_t i = a.tperm ? a.tperm[k] : k;
        tx[t] = __double2float_rn(a.tg[3 * i]);
        ty[t] = __double2float_rn(a.tg[3 * i + 1]);
        tz[t] = __double2float_rn(a.tg[3 * i + 2]);
        tz2[t] = 2.0f * tz[t];
        bl[0] = fminf(bl[0], tx[t]), bl[1] = fminf(bl[1], ty[t]), bl[2] = fminf(bl[2], tz[t]);
        bh[0] = fmaxf(bh[0], tx[t]), bh[1] = fmaxf(bh[1], ty[t]), bh[2] = fmaxf(bh[2], tz[t]);
    }
    // bounding box of the CTA's targets (fminf/fmaxf leave out a NaN coordinate; the pairs of
    // such a target compare false against every threshold, so both loops treat them alike)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            bl[c] = fminf(bl[c], __shfl_xor_sync(0xffffffffu, bl[c], o));
            bh[c] = fmaxf(bh[c], __shfl_xor_sync(0xffffffffu, bh[c], o));
        }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int c = 0; c < 3; c++) s_box[threadIdx.x >> 5][c] = bl[c], s_box[threadIdx.x >> 5][3 + c] = bh[c];
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kF32Threads / 32; w++)
#pragma unroll
        for (int c = 0; c < 3; c++) bl[c] = fminf(bl[c], s_box[w][c]), bh[c] = fmaxf(bh[c], s_box[w][3 + c]);
    double acc[TPT][OUTW];
#pragma unroll
    for (int t = 0; t < TPT; t++)
#pragma unroll
        for (int c = 0; c < OUTW; c++) acc[t][c] = 0.0;

    const int64_t j0 = (int64_t)blockIdx.y * a.split_len;
    const int64_t j1 = min(a.N, j0 + a.split_len);
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    // register prefetch of this thread's source of the first tile
    float4 pre[NQ];
    {
        const int64_t j = j0 + threadIdx.x;
#pragma unroll
        for (int qd = 0; qd < NQ; qd++) pre[qd] = (j < j1) ? a.packed[j * NQ + qd] : zero4;
    }
    for (int64_t jt = j0; jt < j1; jt += kF32Tile) {
        const int cnt = (int)(j1 - jt < kF32Tile ? j1 - jt : kF32Tile);
        __syncthreads();
#pragma unroll
        for (int qd = 0; qd < NQ; qd++) s_src[threadIdx.x * NQ + qd] = pre[qd];
        if constexpr (PACK) {  // {x, y} {h, e2} {f0, f1} {f2, thr}, each value in both halves
            ulonglong2 *d = s_dup + threadIdx.x * 4;
            d[0] = make_ulonglong2(pk2(pre[0].x, pre[0].x), pk2(pre[0].y, pre[0].y));
            d[1] = make_ulonglong2(pk2(pre[0].z, pre[0].z), pk2(pre[0].w, pre[0].w));
            d[2] = make_ulonglong2(pk2(pre[1].x, pre[1].x), pk2(pre[1].y, pre[1].y));
            d[3] = make_ulonglong2(pk2(pre[1].z, pre[1].z), pk2(pre[1].w, pre[1].w));
        }
        __syncthreads();
        {
            const int64_t j = jt + kF32Tile + threadIdx.x;
#pragma unroll
            for (int qd = 0; qd < NQ; qd++) pre[qd] = (j < j1) ? a.packed[j * NQ + qd] : zero4;
        }
        float u[TPT][OUTW];
#pragma unroll
        for (int t = 0; t < TPT; t++)
#pragma unroll
            for (int c = 0; c < OUTW; c++) u[t][c] = 0.0f;
        // no pair of the tile is near when the gap between the two boxes exceeds every
        // threshold of the tile (QF >= gap^2 up to rounding, which the 2^-10 margin covers);
        // the same decision in every thread of the CTA
        bool far_tile = false;
        if (cnt == kF32Tile) {
            const float4 lo = a.tile_box[2 * (jt / kF32Tile)], hi = a.tile_box[2 * (jt / kF32Tile) + 1];
            const float gx = fmaxf(0.0f, fmaxf(lo.x - bh[0], bl[0] - hi.x));
            const float gy = fmaxf(0.0f, fmaxf(lo.y - bh[1], bl[1] - hi.y));
            const float gz = fmaxf(0.0f, fmaxf(lo.z - bh[2], bl[2] - hi.z));
            far_tile = fmaf(gz, gz, fmaf(gy, gy, gx * gx)) > lo.w * (1.0f + 0x1p-10f);
        }
        if (PACK && far_tile) {
            if constexpr (PACK) {
                constexpr int H = TPT / 2;  // register pairs of targets: (0, 1), (2, 3), ...
                f32x2 tx2[H], ty2[H], tz2p[H], u2[H][3];
#pragma unroll
                for (int h = 0; h < H; h++) {
                    tx2[h] = pk2(tx[2 * h], tx[2 * h + 1]), ty2[h] = pk2(ty[2 * h], ty[2 * h + 1]);
                    tz2p[h] = pk2(tz[2 * h], tz[2 * h + 1]);
                    u2[h][0] = u2[h][1] = u2[h][2] = 0ull;
                }
#pragma unroll 2
                for (int k = 0; k < kF32Tile; k++) {
                    const ulonglong2 a0 = s_dup[4 * k], a1 = s_dup[4 * k + 1], a2 = s_dup[4 * k + 2];
                    const f32x2 f2v = s_dup[4 * k + 3].x;
#pragma unroll
                    for (int h = 0; h < H; h++)
                        wall_far_pair2(tx2[h], ty2[h], tz2p[h], a0.x, a0.y, a1.x, a1.y, a2.x, a2.y, f2v, u2[h]);
                }
#pragma unroll
                for (int h = 0; h < H; h++)
#pragma unroll
                    for (int c = 0; c < 3; c++) u[2 * h][c] = lo2(u2[h][c]), u[2 * h + 1][c] = hi2(u2[h][c]);
            }
        } else if (far_tile) {
#pragma unroll kFarUnroll
            for (int k = 0; k < kF32Tile; k++) {
                const float4 p = s_src[k * NQ];
                const float4 q = s_src[k * NQ + 1];
                const float4 r = NF == 2 ? s_src[k * NQ + (NQ - 1)] : zero4;
#pragma unroll
                for (int t = 0; t < TPT; t++)
                    pair_f32_far<KIND, NF, CK, false>(tx[t], ty[t], tz[t], tz2[t], p, q, r, a.alpha_re, a.alpha_im,
                                                      u[t]);
            }
        } else if (cnt == kF32Tile) {
#pragma unroll 2
            for (int k = 0; k < kF32Tile; k++) {
                const float4 p = s_src[k * NQ];
                const float4 q = s_src[k * NQ + 1];
                const float4 r = NF == 2 ? s_src[k * NQ + (NQ - 1)] : zero4;
#pragma unroll
                for (int t = 0; t < TPT; t++)
                    pair_f32_far<KIND, NF, CK>(tx[t], ty[t], tz[t], tz2[t], p, q, r, a.alpha_re, a.alpha_im, u[t]);
            }
        } else {
            for (int k = 0; k < cnt; k++) {
                const float4 p = s_src[k * NQ];
                const float4 q = s_src[k * NQ + 1];
                const float4 r = NF == 2 ? s_src[k * NQ + (NQ - 1)] : zero4;
#pragma unroll
                for (int t = 0; t < TPT; t++)
                    pair_f32_far<KIND, NF, CK>(tx[t], ty[t], tz[t], tz2[t], p, q, r, a.alpha_re, a.alpha_im, u[t]);
            }
        }
#pragma unroll
        for (int t = 0; t < TPT; t++)
#pragma unroll
            for (int c = 0; c < OUTW; c++) acc[t][c] += (double)(KIND == FLG_WALL ? tz2[t] * u[t][c] : u[t][c]);
    }
#pragma unroll
    for (int t = 0; t < TPT; t++) {
        const int64_t i = base + (int64_t)t * kF32Threads;
        if (i < a.M) {
            double *p = a.partial + ((int64_t)blockIdx.y * a.M + i) * OUTW;
#pragma unroll
            for (int c = 0; c < OUTW; c++) p[c] = acc[t][c];
        }
    }
}

// pack FP64 sources into FP32 float4 slots, slot k holding source order[k] (cell order)
__global__ void pack_geometry_kernel(const double *src, const double *eps, const int *order, int64_t N, int NQ,
                                     float4 *packed) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int64_t j = order[k];
    const double e = eps[j];
    const float e2 = __double2float_rn(e * e);
    packed[k * NQ] = make_float4(__double2float_rn(src[3 * j]), __double2float_rn(src[3 * j + 1]),
                                 __double2float_rn(src[3 * j + 2]), e2);
    packed[k * NQ + 1].w = __fmul_rn(17.0f, e2);  // |d|^2 < 16 eps^2  <=>  QF < 17 eps^2
}

// per 256-source tile of the packed sources: bounding box of the FP32 coordinates and the
// largest threshold, {lo x, y, z, max thr} {hi x, y, z, 0}
__global__ void __launch_bounds__(256) tile_box_kernel(const float4 *packed, int64_t N, int NQ, float4 *box) {
    __shared__ float st[7][8];
    const int64_t k = (int64_t)blockIdx.x * 256 + threadIdx.x;
    float v[7] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY, 0.0f};
    if (k < N) {
        const float4 p = packed[k * NQ];
        v[0] = v[3] = p.x, v[1] = v[4] = p.y, v[2] = v[5] = p.z;
        v[6] = packed[k * NQ + 1].w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int c = 0; c < 7; c++) {
            const float w = __shfl_xor_sync(0xffffffffu, v[c], o);
            v[c] = (c < 3) ? fminf(v[c], w) : fmaxf(v[c], w);
        }
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int c = 0; c < 7; c++) st[c][threadIdx.x >> 5] = v[c];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; w++)
            for (int c = 0; c < 7; c++) v[c] = (c < 3) ? fminf(v[c], st[c][w]) : fmaxf(v[c], st[c][w]);
        box[2 * blockIdx.x] = make_float4(v[0], v[1], v[2], v[6]);
        box[2 * blockIdx.x + 1] = make_float4(v[3], v[4], v[5], 0.0f);
    }
}

// slot k gets the strength of source order[k]; src (wall kernel only): the strengths are
// scaled by the source height z_j, the factor of the wall pair that depends on the source
// alone (see wall_far_geo)
__global__ void pack_strengths_kernel(const double *f, const double *src, const int *order, int64_t N, int NF,
                                      float4 *packed) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int64_t j = order[k];
    const int NQ = 1 + NF;
    float4 *q = packed + k * NQ + 1;
    const double *fj = f + (int64_t)3 * NF * j;
    const double h = src ? src[3 * j + 2] : 1.0;
    if (NF == 1) {
        q->x = __double2float_rn(h * fj[0]);
        q->y = __double2float_rn(h * fj[1]);
        q->z = __double2float_rn(h * fj[2]);
    } else {  // interleaved complex (re, im) per component
        q->x = __double2float_rn(h * fj[0]);
        q->y = __double2float_rn(h * fj[2]);
        q->z = __double2float_rn(h * fj[4]);
        q[1] = make_float4(__double2float_rn(h * fj[1]), __double2float_rn(h * fj[3]), __double2float_rn(h * fj[5]),
                           0.0f);
    }
}

// ---------------------------------------------------------------------------
// cell list for the near field
// ---------------------------------------------------------------------------
__global__ void cell_bounds_kernel(const double *src, const double *eps, int64_t N, double *blk) {
    __shared__ double sm[7][256];
    double v[7] = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300, 0.0};
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
        for (int c = 0; c < 3; c++) {
            double x = src[3 * j + c];
            v[c] = fmin(v[c], x);
            v[3 + c] = fmax(v[3 + c], x);
        }
        v[6] = fmax(v[6], fabs(eps[j]));
    }
    for (int c = 0; c < 7; c++) sm[c][threadIdx.x] = v[c];
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            for (int c = 0; c < 3; c++) sm[c][threadIdx.x] = fmin(sm[c][threadIdx.x], sm[c][threadIdx.x + w]);
            for (int c = 3; c < 7; c++) sm[c][threadIdx.x] = fmax(sm[c][threadIdx.x], sm[c][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int c = 0; c < 7; c++) blk[blockIdx.x * 7 + c] = sm[c][0];
}

__global__ void cell_setup_kernel(const double *blk, int nblk, CellGrid *g) {
    if (threadIdx.x != 0) return;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300}, emax = 0.0;
    for (int b = 0; b < nblk; b++) {
        for (int c = 0; c < 3; c++) {
            lo[c] = fmin(lo[c], blk[b * 7 + c]);
            hi[c] = fmax(hi[c], blk[b * 7 + 3 + c]);
        }
        emax = fmax(emax, blk[b * 7 + 6]);
    }
    // cell edge >= 4.2 max eps: every pair with r < 4 eps (plus FP32 rounding)
    // lies in the 27-cell neighbourhood of the target's cell
    double h = fmax(4.2 * emax, 1e-300);
    double ext[3];
    for (int c = 0; c < 3; c++) ext[c] = fmax(hi[c] - lo[c], 0.0);
    for (int it = 0; it < 64; it++) {
        double cells = 1.0;
        for (int c = 0; c < 3; c++) cells *= floor(ext[c] / h) + 1.0;
        if (cells <= (double)kMaxCells) break;
        h *= fmax(1.01, cbrt(cells / (double)kMaxCells));
    }
    double n[3];
    for (int c = 0; c < 3; c++) n[c] = floor(ext[c] / h) + 1.0;
    const bool ok = n[0] >= 1.0 && n[1] >= 1.0 && n[2] >= 1.0 && n[0] * n[1] * n[2] <= (double)kMaxCells &&
                    h > 0.0 && h < 1e300 && lo[0] == lo[0] && lo[1] == lo[1] && lo[2] == lo[2];
    if (!ok) {  // non-finite input: one cell holding every source (still exact, only slower)
        h = INFINITY;
        n[0] = n[1] = n[2] = 1.0;
        lo[0] = lo[1] = lo[2] = 0.0;
    }
    g->h = h;
    g->inv_h = ok ? 1.0 / h : 0.0;
    g->ox = lo[0];
    g->oy = lo[1];
    g->oz = lo[2];
    g->nx = (int)n[0];
    g->ny = (int)n[1];
    g->nz = (int)n[2];
    g->ncell = g->nx * g->ny * g->nz;
}

__device__ __forceinline__ int cell_coord(double x, double o, double inv_h, int n) {
    double c = floor((x - o) * inv_h);
    c = fmin(fmax(c, 0.0), (double)(n - 1));
    return (int)c;
}

__global__ void cell_count_kernel(const double *src, int64_t N, const CellGrid *g, int *cell_of, int *counts) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    const CellGrid G = *g;
    int cx = cell_coord(src[3 * j], G.ox, G.inv_h, G.nx);
    int cy = cell_coord(src[3 * j + 1], G.oy, G.inv_h, G.ny);
    int cz = cell_coord(src[3 * j + 2], G.oz, G.inv_h, G.nz);
    int c = (cz * G.ny + cy) * G.nx + cx;
    cell_of[j] = c;
    atomicAdd(&counts[c], 1);
}

// exclusive scan of counts[0..kMaxCells) -> offsets[0..kMaxCells], two levels
__global__ void scan_block_kernel(const int *in, int *out, int *block_sums, int n) {
    __shared__ int sm[kScanBlock];
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    int v = i < n ? in[i] : 0;
    sm[threadIdx.x] = v;
    __syncthreads();
    for (int w = 1; w < kScanBlock; w <<= 1) {
        int t = (int)threadIdx.x >= w ? sm[threadIdx.x - w] : 0;
        __syncthreads();
        sm[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sm[threadIdx.x] - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = sm[threadIdx.x];
}

__global__ void scan_sums_kernel(int *block_sums, int nb) {
    __shared__ int sm[kScanBlock];
    const int t = threadIdx.x;
    int v = t < nb ? block_sums[t] : 0;
    sm[t] = v;
    __syncthreads();
    for (int w = 1; w < kScanBlock; w <<= 1) {
        int x = t >= w ? sm[t - w] : 0;
        __syncthreads();
        sm[t] += x;
        __syncthreads();
    }
    if (t < nb) block_sums[t] = sm[t] - v;
    if (t == kScanBlock - 1) block_sums[nb] = sm[t];  // grand total
}

__global__ void scan_add_kernel(int *out, const int *block_sums, int n) {
    const int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_sums[blockIdx.x];
}

__global__ void scan_total_kernel(int *out, const int *block_sums, int nb, int n) { out[n] = block_sums[nb]; }

__global__ void cell_scatter_kernel(const int *cell_of, int64_t N, const int *offsets, int *cursor, int *sorted) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    int c = cell_of[j];
    int pos = offsets[c] + atomicAdd(&cursor[c], 1);
    sorted[pos] = (int)j;
}

// deterministic order within each cell: ascending source index
__global__ void cell_sort_kernel(const int *offsets, const CellGrid *g, int *sorted) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g->ncell) return;
    const int b = offsets[c], e = offsets[c + 1];
    for (int k = b + 1; k < e; k++) {
        int v = sorted[k];
        int m = k - 1;
        while (m >= b && sorted[m] > v) {
            sorted[m + 1] = sorted[m];
            m--;
        }
        sorted[m + 1] = v;
    }
}

struct NearArgs {
    const double *tg;
    int64_t M;
    const int *tperm;  // processing position -> target index (null: identity), as in the far field
    const double *src;
    const double *eps;
    const double *f;
    int64_t N;
    const float4 *packed;
    int NQ;
    const CellGrid *grid;
    const int *offsets;
    const int *sorted;
    double alpha_re, alpha_im;
    FinalArgs fin;
};

template <int KIND, int NF, bool CK>
__global__ void __launch_bounds__(128) near_f64_kernel(NearArgs a) {
    constexpr int OUTW = (NF == 2 || CK) ? 6 : 3;
    const int64_t kt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // processing position
    if (kt >= a.M) return;
    const int64_t i = a.tperm ? a.tperm[kt] : kt;
    const CellGrid G = *a.grid;
    const double tx = a.tg[3 * i], ty = a.tg[3 * i + 1], tz = a.tg[3 * i + 2], tz2 = 2.0 * tz;
    const float fx = __double2float_rn(tx), fy = __double2float_rn(ty), fz = __double2float_rn(tz);
    double u[OUTW];
#pragma unroll
    for (int c = 0; c < OUTW; c++) u[c] = 0.0;
    // far partials, summed in split order
    for (int s = 0; s < a.fin.S; s++) {
        const double *p = a.fin.partial + ((int64_t)s * a.M + kt) * OUTW;
#pragma unroll
        for (int c = 0; c < OUTW; c++) u[c] += p[c];
    }
    const int cx = cell_coord(tx, G.ox, G.inv_h, G.nx);
    const int cy = cell_coord(ty, G.oy, G.inv_h, G.ny);
    const int cz = cell_coord(tz, G.oz, G.inv_h, G.nz);
    // a target more than one cell outside the source box has no near pair
    const bool outside = (tx - G.ox) * G.inv_h < -1.0 || (ty - G.oy) * G.inv_h < -1.0 ||
                         (tz - G.oz) * G.inv_h < -1.0 || (tx - G.ox) * G.inv_h > G.nx + 1.0 ||
                         (ty - G.oy) * G.inv_h > G.ny + 1.0 || (tz - G.oz) * G.inv_h > G.nz + 1.0;
    if (!outside) {
        for (int z = max(cz - 1, 0); z <= min(cz + 1, G.nz - 1); z++)
            for (int y = max(cy - 1, 0); y <= min(cy + 1, G.ny - 1); y++)
                for (int x = max(cx - 1, 0); x <= min(cx + 1, G.nx - 1); x++) {
                    const int c = (z * G.ny + y) * G.nx + x;
                    const int b = a.offsets[c], e = a.offsets[c + 1];
                    for (int k = b; k < e; k++) {
                        const int j = a.sorted[k];
                        const float4 p = a.packed[(int64_t)k * a.NQ];  // packed in cell order
                        const float thr = a.packed[(int64_t)k * a.NQ + 1].w;
                        const float d0 = sub_rn(fx, p.x), d1 = sub_rn(fy, p.y), d2 = sub_rn(fz, p.z);
                        if (free_Q_f32(d0, d1, d2, p.w) < thr) {
                            const double ej = a.eps[j];
                            double fj[3 * NF];
                            load_strength<NF>(a.f, j, fj);
                            pair_f64<KIND, NF, CK>(tx, ty, tz, tz2, a.src[3 * j], a.src[3 * j + 1], a.src[3 * j + 2],
                                                   ej * ej, fj, a.alpha_re, a.alpha_im, u);
                        }
                    }
                }
    }
    final_store(a.fin, i, u);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static void mu_division(double mu_re, double mu_im, FinalArgs &f) {
    f.mu_complex = mu_im != 0.0;
    f.mu_re = mu_re;
    if (f.mu_complex) {
        // numpy's complex division (Smith's method)
        if (fabs(mu_re) >= fabs(mu_im)) {
            f.mu_branch = 0;
            f.mu_rat = mu_im / mu_re;
            f.mu_scl = 1.0 / (mu_re + mu_im * f.mu_rat);
        } else {
            f.mu_branch = 1;
            f.mu_rat = mu_re / mu_im;
            f.mu_scl = 1.0 / (mu_im + mu_re * f.mu_rat);
        }
    }
}

static void split_plan(int64_t M, int64_t N, int targets_per_cta, int tile, int ctas_per_sm, int64_t &S,
                       int64_t &split_len) {
    if (N <= 0) {
        S = 0;
        split_len = 0;
        return;
    }
    const int64_t mblocks = ceil_div(M, targets_per_cta);
    const int64_t want = 4LL * sm_count() * ctas_per_sm;
    S = std::max<int64_t>(1, ceil_div(want, mblocks));
    S = std::min<int64_t>(S, ceil_div(N, tile));
    S = std::min<int64_t>(S, 4096);
    split_len = ceil_div(ceil_div(N, S), tile) * tile;
    S = ceil_div(N, split_len);
}

// targets per thread of the FP32 far-field kernel for real strengths and kernels
#ifndef FLG_FAR_TPT
#define FLG_FAR_TPT 2
#endif
static inline int far_tpt(int kind, int nf, bool ck) { return (nf == 1 && !ck) ? FLG_FAR_TPT : 1; }

void sum_layout(int kind, int64_t M, int64_t N, int nf, bool ck, int precision, SumLayout &L) {
    L.nf = nf;
    L.ck = ck;
    L.outw = out_width(nf, ck);
    L.NQ = 1 + nf;
    if (precision == FLG_PREC_FP64) {
        split_plan(M, N, kF64Threads, kF64Tile, 8, L.S, L.split_len);
    } else {
        split_plan(M, N, kF32Threads * far_tpt(kind, nf, ck), kF32Tile, 4, L.S, L.split_len);
    }
}

template <class A>
static void carve_plan(A &ar, int64_t M, int64_t N, const SumLayout &L, int precision, SumPlan *p) {
    p->partial = ar.template take<double>((size_t)std::max<int64_t>(L.S, 1) * M * L.outw);
    if (precision == FLG_PREC_MIXED) {
        p->packed = ar.template take<float4>((size_t)N * L.NQ);
        p->tile_box = ar.template take<float4>(2 * (size_t)ceil_div(std::max<int64_t>(N, 1), kF32Tile));
        p->grid = ar.template take<CellGrid>(1);
        p->bounds = ar.template take<double>(kBoundBlocks * 7);
        p->cell_of = ar.template take<int>(N);
        p->counts = ar.template take<int>(kMaxCells);
        p->offsets = ar.template take<int>(kMaxCells + 1);
        p->block_sums = ar.template take<int>(kMaxCells / kScanBlock + 1);
        p->sorted = ar.template take<int>(N);
        p->tcell = p->toffsets = p->tperm = nullptr;
        if (M >= kSortTargetsMin) {
            p->tcell = ar.template take<int>(M);
            p->toffsets = ar.template take<int>(kMaxCells + 1);
            p->tperm = ar.template take<int>(M);
        }
    }
}

size_t sum_workspace_bytes(int kind, int64_t M, int64_t N, int nf, bool ck, int precision) {
    SumLayout L;
    sum_layout(kind, M, N, nf, ck, precision, L);
    CountingArena sz;
    SumPlan p;
    carve_plan(sz, M, N, L, precision, &p);
    return sz.bytes();
}

int sum_plan_carve(void *work, size_t work_bytes, int64_t M, int64_t N, const SumLayout &L, int precision,
                   SumPlan *p) {
    if (M == 0 || N == 0) return FLG_OK;
    Arena ar(work, work_bytes);
    carve_plan(ar, M, N, L, precision, p);
    const bool ok = p->partial != nullptr && (precision != FLG_PREC_MIXED || p->sorted != nullptr) &&
                    (precision != FLG_PREC_MIXED || M < kSortTargetsMin || p->tperm != nullptr);
    FLG_REQUIRE(ok, "workspace too small: %zu bytes given, %zu needed", work_bytes,
                sum_workspace_bytes(0, M, N, L.nf, L.ck, precision));
    return FLG_OK;
}

// Geometry part of the mixed plan (sources and eps only): packed FP32
// coordinates and the sorted cell list.  Reusable while the sources stay put.
int sum_plan_geometry(const double *src, const double *eps, int64_t N, const SumLayout &L, SumPlan *p,
                      cudaStream_t st) {
    if (N == 0) return FLG_OK;
    const int tb = 256;
    cell_bounds_kernel<<<kBoundBlocks, 256, 0, st>>>(src, eps, N, p->bounds);
    FLG_LAUNCH_CHECK();
    cell_setup_kernel<<<1, 32, 0, st>>>(p->bounds, kBoundBlocks, p->grid);
    FLG_LAUNCH_CHECK();
    FLG_CUDA(cudaMemsetAsync(p->counts, 0, sizeof(int) * kMaxCells, st));
    cell_count_kernel<<<(unsigned)ceil_div(N, tb), tb, 0, st>>>(src, N, p->grid, p->cell_of, p->counts);
    FLG_LAUNCH_CHECK();
    const int nb = kMaxCells / kScanBlock;
    scan_block_kernel<<<nb, kScanBlock, 0, st>>>(p->counts, p->offsets, p->block_sums, kMaxCells);
    FLG_LAUNCH_CHECK();
    scan_sums_kernel<<<1, kScanBlock, 0, st>>>(p->block_sums, nb);
    FLG_LAUNCH_CHECK();
    scan_add_kernel<<<nb, kScanBlock, 0, st>>>(p->offsets, p->block_sums, kMaxCells);
    FLG_LAUNCH_CHECK();
    scan_total_kernel<<<1, 1, 0, st>>>(p->offsets, p->block_sums, nb, kMaxCells);
    FLG_LAUNCH_CHECK();
    FLG_CUDA(cudaMemsetAsync(p->counts, 0, sizeof(int) * kMaxCells, st));
    cell_scatter_kernel<<<(unsigned)ceil_div(N, tb), tb, 0, st>>>(p->cell_of, N, p->offsets, p->counts, p->sorted);
    FLG_LAUNCH_CHECK();
    cell_sort_kernel<<<kMaxCells / 256, 256, 0, st>>>(p->offsets, p->grid, p->sorted);
    FLG_LAUNCH_CHECK();
    // the FP32 sources in cell order, and the bounding box of each far-field tile of them
    pack_geometry_kernel<<<(unsigned)ceil_div(N, tb), tb, 0, st>>>(src, eps, p->sorted, N, L.NQ, p->packed);
    FLG_LAUNCH_CHECK();
    tile_box_kernel<<<(unsigned)ceil_div(N, kF32Tile), 256, 0, st>>>(p->packed, N, L.NQ, p->tile_box);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

// Processing order of a large target set: bucketed by the cell of the source grid they fall
// in (a counting sort; the order within a cell does not matter, since a target's sum does
// not depend on which CTA computes it).  Reuses the counting buffers of the source cell
// list, which sum_plan_geometry no longer needs.
static int sort_targets(const double *tg, int64_t M, const SumPlan *p, cudaStream_t st) {
    const int tb = 256;
    FLG_CUDA(cudaMemsetAsync(p->counts, 0, sizeof(int) * kMaxCells, st));
    cell_count_kernel<<<(unsigned)ceil_div(M, tb), tb, 0, st>>>(tg, M, p->grid, p->tcell, p->counts);
    FLG_LAUNCH_CHECK();
    const int nb = kMaxCells / kScanBlock;
    scan_block_kernel<<<nb, kScanBlock, 0, st>>>(p->counts, p->toffsets, p->block_sums, kMaxCells);
    FLG_LAUNCH_CHECK();
    scan_sums_kernel<<<1, kScanBlock, 0, st>>>(p->block_sums, nb);
    FLG_LAUNCH_CHECK();
    scan_add_kernel<<<nb, kScanBlock, 0, st>>>(p->toffsets, p->block_sums, kMaxCells);
    FLG_LAUNCH_CHECK();
    FLG_CUDA(cudaMemsetAsync(p->counts, 0, sizeof(int) * kMaxCells, st));
    cell_scatter_kernel<<<(unsigned)ceil_div(M, tb), tb, 0, st>>>(p->tcell, M, p->toffsets, p->counts, p->tperm);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

template <int KIND, int NF, bool CK>
static int launch_sum(const SumRun &r, const SumLayout &L, int precision, const SumPlan *p, cudaStream_t st) {
    FinalArgs fin{};
    fin.partial = p->partial;
    fin.S = (int)L.S;
    fin.M = r.M;
    fin.outw = L.outw;
    fin.scale = (KIND == FLG_BRINKMANLET) ? 1.0 / (4.0 * kPi) : 1.0 / (8.0 * kPi);
    fin.out_complex = r.out_complex;
    mu_division(r.mu_re, r.mu_im, fin);
    fin.out = r.out;
    if (r.M == 0) return FLG_OK;
    if (precision == FLG_PREC_FP64 || r.N == 0) {
        if (r.N > 0) {
            SumArgs a{r.tg, r.M, r.src, r.eps, r.f, r.N, L.split_len, r.alpha_re, r.alpha_im, p->partial};
            dim3 grid((unsigned)ceil_div(r.M, kF64Threads), (unsigned)L.S);
            prof_begin(FLG_SLOT_SUM_F64, st);
            sum_f64_kernel<KIND, NF, CK><<<grid, kF64Threads, 0, st>>>(a);
            FLG_LAUNCH_CHECK();
            prof_end(FLG_SLOT_SUM_F64, st);
        } else {
            fin.S = 0;
        }
        finalize_kernel<<<(unsigned)ceil_div(r.M, 256), 256, 0, st>>>(fin);
        FLG_LAUNCH_CHECK();
        return FLG_OK;
    }
    // mixed: strengths into the packed slots, FP32 far field, FP64 near field + combine
    pack_strengths_kernel<<<(unsigned)ceil_div(r.N, 256), 256, 0, st>>>(r.f, KIND == FLG_WALL ? r.src : nullptr,
                                                                       p->sorted, r.N, NF, p->packed);
    FLG_LAUNCH_CHECK();
    // targets in cell order: the sources' own order when the targets are the sources, a
    // bucket sort for other large target sets, the given order for small ones
    const int *tperm = nullptr;
    if (r.tg == r.src && r.M == r.N) {
        tperm = p->sorted;
    } else if (r.M >= kSortTargetsMin && p->tperm) {
        FLG_TRY(sort_targets(r.tg, r.M, p, st));
        tperm = p->tperm;
    }
    constexpr int TPT = (NF == 1 && !CK) ? FLG_FAR_TPT : 1;
    FarArgs fa{r.tg, r.M, tperm, p->packed, p->tile_box, r.N, L.split_len, (float)r.alpha_re, (float)r.alpha_im,
               p->partial};
    dim3 grid((unsigned)ceil_div(r.M, kF32Threads * TPT), (unsigned)L.S);
    prof_begin(FLG_SLOT_FAR_F32, st);
    far_f32_kernel<KIND, NF, CK, TPT><<<grid, kF32Threads, 0, st>>>(fa);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_FAR_F32, st);
    NearArgs na{r.tg, r.M, tperm, r.src, r.eps, r.f, r.N, p->packed, L.NQ, p->grid, p->offsets, p->sorted,
                r.alpha_re, r.alpha_im, fin};
    prof_begin(FLG_SLOT_NEAR_F64, st);
    near_f64_kernel<KIND, NF, CK><<<(unsigned)ceil_div(r.M, 128), 128, 0, st>>>(na);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_NEAR_F64, st);
    return FLG_OK;
}

int sum_run(const SumRun &r, const SumLayout &L, int precision, const SumPlan *p, cudaStream_t st) {
    const int nf = L.nf;
    const bool ck = L.ck;
    switch (r.kind) {
        case FLG_STOKESLET:
            return nf == 1 ? launch_sum<FLG_STOKESLET, 1, false>(r, L, precision, p, st)
                           : launch_sum<FLG_STOKESLET, 2, false>(r, L, precision, p, st);
        case FLG_WALL:
            return nf == 1 ? launch_sum<FLG_WALL, 1, false>(r, L, precision, p, st)
                           : launch_sum<FLG_WALL, 2, false>(r, L, precision, p, st);
        case FLG_BRINKMANLET:
            if (ck)
                return nf == 1 ? launch_sum<FLG_BRINKMANLET, 1, true>(r, L, precision, p, st)
                               : launch_sum<FLG_BRINKMANLET, 2, true>(r, L, precision, p, st);
            return nf == 1 ? launch_sum<FLG_BRINKMANLET, 1, false>(r, L, precision, p, st)
                           : launch_sum<FLG_BRINKMANLET, 2, false>(r, L, precision, p, st);
    }
    set_error("unknown kernel kind %d", r.kind);
    return FLG_ERR_INVALID;
}

int check_kernel_args(int kind, double alpha_re, double alpha_im) {
    FLG_REQUIRE(kind == FLG_STOKESLET || kind == FLG_WALL || kind == FLG_BRINKMANLET, "unknown kernel kind %d",
                kind);
    if (kind == FLG_BRINKMANLET) {
        FLG_REQUIRE(alpha_re == alpha_re && alpha_im == alpha_im, "alpha must be finite");
        FLG_REQUIRE(alpha_re >= 0.0, "alpha must have a non-negative real part");
    }
    return FLG_OK;
}

}  // namespace flg

using namespace flg;

extern "C" size_t flg_evaluate_workspace(int kind, int64_t M, int64_t N, int strengths_complex, double alpha_im,
                                         int precision) {
    if (M < 0 || N < 0) return 0;
    const bool ck = kind == FLG_BRINKMANLET && alpha_im != 0.0;
    return sum_workspace_bytes(kind, M, N, strengths_complex ? 2 : 1, ck, precision);
}

extern "C" int flg_evaluate(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                            const double *sources, const double *eps, int64_t N, const double *strengths,
                            int strengths_complex, double mu_re, double mu_im, double *out, int precision,
                            void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_evaluate");
    FLG_TRY(check_kernel_args(kind, alpha_re, alpha_im));
    FLG_REQUIRE(M >= 0 && N >= 0, "negative sizes M=%lld N=%lld", (long long)M, (long long)N);
    FLG_REQUIRE(precision == FLG_PREC_FP64 || precision == FLG_PREC_MIXED, "unknown precision %d", precision);
    FLG_REQUIRE(M < (1LL << 31) && N < (1LL << 31), "at most 2^31 - 1 targets and sources");
    FLG_REQUIRE(!(mu_re == 0.0 && mu_im == 0.0), "mu must be non-zero");
    FLG_REQUIRE(M == 0 || (targets && out), "null targets/out");
    FLG_REQUIRE(N == 0 || (sources && eps && strengths), "null sources/eps/strengths");
    const bool ck = kind == FLG_BRINKMANLET && alpha_im != 0.0;
    const int nf = strengths_complex ? 2 : 1;
    SumLayout L;
    sum_layout(kind, M, N, nf, ck, precision, L);
    SumPlan p{};
    FLG_TRY(sum_plan_carve(work, work_bytes, M, N, L, precision, &p));
    cudaStream_t st = as_stream(stream);
    if (precision == FLG_PREC_MIXED && M > 0 && N > 0) FLG_TRY(sum_plan_geometry(sources, eps, N, L, &p, st));
    SumRun r{};
    r.kind = kind;
    r.tg = targets;
    r.M = M;
    r.src = sources;
    r.eps = eps;
    r.f = strengths;
    r.N = N;
    r.alpha_re = alpha_re;
    r.alpha_im = alpha_im;
    r.mu_re = mu_re;
    r.mu_im = mu_im;
    r.out = out;
    r.out_complex = (strengths_complex || ck || mu_im != 0.0) ? 1 : 0;
    return sum_run(r, L, precision, &p, st);
}

// ---------------------------------------------------------------------------
// Allocation-free FP64 sum (flg_evaluate_noalloc).
//
// Some callers cannot allocate device memory at all: a host application that
// reserves the whole GPU for its own memory pool at start-up, or a plug-in
// running inside a framework that forbids cudaMalloc once it is running.
// They cannot provide the workspace flg_evaluate asks for either, so this
// variant keeps the only scratch the FP64 sum needs -- the per-split partial
// sums -- in the fixed-size device array below.  The array exists once per
// GPU that loads the library and stays allocated until the process exits.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_addr[kMaxDevices] = {};
}  // namespace

// Device address of g_noalloc_scratch on the current device.  In host code the
// array's name is only a host-side stand-in, so the address is looked up once
// per device (with that device current) and cached.
static int noalloc_scratch(void **addr) {
    int dev = 0;
    FLG_CUDA(cudaGetDevice(&dev));
    FLG_REQUIRE(dev >= 0 && dev < kMaxDevices, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (g_noalloc_addr[dev] == nullptr) {
        void *p = nullptr;
        FLG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_addr[dev] = p;
    }
    *addr = g_noalloc_addr[dev];
    return FLG_OK;
}

extern "C" size_t flg_evaluate_noalloc_max_bytes(void) { return kNoAllocScratchBytes; }

extern "C" int flg_evaluate_noalloc(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                                    const double *sources, const double *eps, int64_t N, const double *strengths,
                                    int strengths_complex, double mu_re, double mu_im, double *out, void *stream) {
    FLG_TRY(check_kernel_args(kind, alpha_re, alpha_im));
    FLG_REQUIRE(M >= 0 && N >= 0, "negative sizes M=%lld N=%lld", (long long)M, (long long)N);
    FLG_REQUIRE(M < (1LL << 31) && N < (1LL << 31), "at most 2^31 - 1 targets and sources");
    FLG_REQUIRE(!(mu_re == 0.0 && mu_im == 0.0), "mu must be non-zero");
    const bool ck = kind == FLG_BRINKMANLET && alpha_im != 0.0;
    const int nf = strengths_complex ? 2 : 1;
    SumLayout L;
    sum_layout(kind, M, N, nf, ck, FLG_PREC_FP64, L);
    // one partial sum per (split, target): shrink the number of source splits
    // until they fit the fixed array; one split is the minimum
    const size_t per_split = (size_t)M * L.outw * sizeof(double);
    FLG_REQUIRE(per_split <= kNoAllocScratchBytes,
                "flg_evaluate_noalloc: %lld targets need %zu bytes of scratch, more than its fixed %zu; "
                "use flg_evaluate with a workspace",
                (long long)M, per_split, kNoAllocScratchBytes);
    if (M == 0) return FLG_OK;
    FLG_REQUIRE(targets && out, "null targets/out");
    FLG_REQUIRE(N == 0 || (sources && eps && strengths), "null sources/eps/strengths");
    if (N > 0 && (size_t)L.S * per_split > kNoAllocScratchBytes) {
        const int64_t smax = (int64_t)(kNoAllocScratchBytes / per_split);
        L.split_len = ceil_div(ceil_div(N, smax), kF64Tile) * kF64Tile;
        L.S = ceil_div(N, L.split_len);
    }
    SumPlan p{};
    FLG_TRY(noalloc_scratch((void **)&p.partial));
    SumRun r{};
    r.kind = kind;
    r.tg = targets;
    r.M = M;
    r.src = sources;
    r.eps = eps;
    r.f = strengths;
    r.N = N;
    r.alpha_re = alpha_re;
    r.alpha_im = alpha_im;
    r.mu_re = mu_re;
    r.mu_im = mu_im;
    r.out = out;
    r.out_complex = (strengths_complex || ck || mu_im != 0.0) ? 1 : 0;
    // every partial that is read is written earlier in the same call: nothing to clear
    return sum_run(r, L, FLG_PREC_FP64, &p, as_stream(stream));
}
