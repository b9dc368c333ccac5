// assemble.cu -- dense mobility matrices and dense helpers.
//
//  flg_assemble            fluidlets.assemble (core/assemble.py:27-46, _fill 15-24)
//  flg_assemble_self_uniform  the same for targets = sources and one blob width (half
//                          the pair evaluations: the matrix is symmetric)
//  flg_assemble_nearest    fluidlets.assemble_nearest (core/assemble.py:68-101,
//                          _fill_nearest 49-58), deterministic segmented sum
//  flg_swimmer_constraints the rows/columns of swimming.py:90-99
//  flg_gemv_f64, flg_convert_f64_f32
//
// Assembly writes K / mu once, directly in the requested element type (the
// reference makes two extra full copies, core/assemble.py:46).  Each thread
// computes one 3x3 block G(x_i, y_j) in FP64 and stores its nine entries;
// consecutive threads take consecutive sources j, so a warp writes three
// contiguous 96-element row segments.
#include <cuda_bf16.h>

#include "flg_common.cuh"
#include "pair_math.cuh"
#include "sum_plan.cuh"

namespace flg {

struct AsmArgs {
    const double *tg;
    int64_t M;
    const double *src;
    const double *eps;
    int64_t N;
    double are, aim;
    double scale;  // global kernel scale
    // 1/mu as a complex number
    double imu_re, imu_im;
    void *out;
    int out_type;
    int64_t ld;
    int64_t col_off;  // first column written (nearest: group index scale)
    int64_t sys_stride;  // bucket batches: elements between the outputs of consecutive systems
};

// 3x3 block (row-major, before scale / mu); complex part only for complex alpha
template <int KIND, bool CK>
__device__ __forceinline__ void block_f64(double tx, double ty, double tz, double sx, double sy, double sz,
                                          double e2, double are, double aim, double G[9], double Gi[9]) {
    if constexpr (KIND == FLG_WALL) {
        WallGeo<double> g = wall_geo<double, false>(tx, ty, tz, 2.0 * tz, sx, sy, sz, e2, 0.0);
        const double W = g.W2, Zs = g.Z3 + g.s5x3;
        const double dd[2] = {g.d0, g.d1};
        for (int j = 0; j < 2; j++) {
            G[3 * j + 0] = W * fma(dd[j] * g.d0, Zs, j == 0 ? g.cxy : 0.0);
            G[3 * j + 1] = W * fma(dd[j] * g.d1, Zs, j == 1 ? g.cxy : 0.0);
            G[3 * j + 2] = W * dd[j] * fma(g.Z3, g.dm, -g.s5x3 * g.dp);
        }
        const double c2 = fma(g.dm, g.Z3, g.s5x3 * g.dp);
        G[6] = W * g.d0 * c2;
        G[7] = W * g.d1 * c2;
        G[8] = W * fma(g.dm * g.dm, g.Z3, fma(-g.s5x3 * g.dp, g.dp, g.cz));
    } else {
        const double d[3] = {tx - sx, ty - sy, tz - sz};
        const double Q = fma(d[2], d[2], fma(d[1], d[1], fma(d[0], d[0], e2)));
        const double s = rsq(Q);
        if constexpr (CK) {
            cpx<double> A, B;
            brink_AB_c<double>(s, Q, e2, are, aim, A, B);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) {
                    G[3 * a + b] = fma(B.re * d[a], d[b], a == b ? A.re : 0.0);
                    Gi[3 * a + b] = fma(B.im * d[a], d[b], a == b ? A.im : 0.0);
                }
            return;
        } else {
            double A, B;
            if constexpr (KIND == FLG_STOKESLET) stokeslet_AB(s, e2, A, B);
            else brink_AB<double>(s, Q, e2, are, A, B);
            for (int a = 0; a < 3; a++)
                for (int b = 0; b < 3; b++) G[3 * a + b] = fma(B * d[a], d[b], a == b ? A : 0.0);
        }
    }
    if constexpr (CK == false)
        for (int k = 0; k < 9; k++) Gi[k] = 0.0;
}

__device__ __forceinline__ void store_block(const AsmArgs &a, int64_t i, int64_t col, const double G[9],
                                            const double Gi[9], bool cplx) {
    for (int r = 0; r < 3; r++) {
        const int64_t row = 3 * i + r;
        for (int c = 0; c < 3; c++) {
            const int64_t off = row * a.ld + col + c;
            // (G + i Gi) * scale * (1/mu)
            const double gr = G[3 * r + c] * a.scale, gi = cplx ? Gi[3 * r + c] * a.scale : 0.0;
            const double vr = gr * a.imu_re - gi * a.imu_im;
            const double vi = gr * a.imu_im + gi * a.imu_re;
            switch (a.out_type) {
                case FLG_F64: ((double *)a.out)[off] = vr; break;
                case FLG_C128:
                    ((double *)a.out)[2 * off] = vr;
                    ((double *)a.out)[2 * off + 1] = vi;
                    break;
                case FLG_F32: ((float *)a.out)[off] = (float)vr; break;
                default: ((__nv_bfloat16 *)a.out)[off] = __double2bfloat16(vr); break;
            }
        }
    }
}

template <int KIND, bool CK>
__global__ void __launch_bounds__(128) assemble_kernel(AsmArgs a) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.N) return;
    const double sx = a.src[3 * j], sy = a.src[3 * j + 1], sz = a.src[3 * j + 2];
    const double e = a.eps[j], e2 = e * e;
    const bool cplx = CK || a.imu_im != 0.0;
    for (int64_t i = blockIdx.y; i < a.M; i += gridDim.y) {
        double G[9], Gi[9];
        block_f64<KIND, CK>(a.tg[3 * i], a.tg[3 * i + 1], a.tg[3 * i + 2], sx, sy, sz, e2, a.are, a.aim, G, Gi);
        store_block(a, i, 3 * j, G, Gi, cplx);
    }
}

// Self-assembly (targets = sources) with one blob width: the matrix is symmetric.  For the
// free kernels block (j, i) equals block (i, j) bit for bit (d -> -d is exact and the block
// depends on d only through products d_a d_b and |d|^2), so the mirror is written as is; for
// the wall kernel it is the transpose (Lorentz reciprocity of the image system, equal to
// rounding).  Thread j takes targets i <= j in tiles of kSymTile rows: it writes block (i, j)
// (a warp covers contiguous row segments) and its mirror at (j, i) (per thread, three row
// segments of 3 kSymTile entries per tile); half the pair evaluations of assemble_kernel.
constexpr int kSymTile = 8;
template <int KIND, bool CK, bool TRANSPOSE>
__global__ void __launch_bounds__(128) assemble_sym_kernel(AsmArgs a, double e2) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.N) return;
    const double sx = a.src[3 * j], sy = a.src[3 * j + 1], sz = a.src[3 * j + 2];
    const bool cplx = CK || a.imu_im != 0.0;
    for (int64_t i0 = (int64_t)blockIdx.y * kSymTile; i0 <= j; i0 += (int64_t)gridDim.y * kSymTile) {
        for (int t = 0; t < kSymTile; t++) {
            const int64_t i = i0 + t;
            if (i > j) break;
            double G[9], Gi[9];
            block_f64<KIND, CK>(a.src[3 * i], a.src[3 * i + 1], a.src[3 * i + 2], sx, sy, sz, e2, a.are, a.aim, G,
                                Gi);
            store_block(a, i, 3 * j, G, Gi, cplx);
            if (i == j) continue;
            if (TRANSPOSE) {
#pragma unroll
                for (int r = 0; r < 3; r++)
#pragma unroll
                    for (int c = r + 1; c < 3; c++) {
                        const double u = G[3 * r + c], v = Gi[3 * r + c];
                        G[3 * r + c] = G[3 * c + r], Gi[3 * r + c] = Gi[3 * c + r];
                        G[3 * c + r] = u, Gi[3 * c + r] = v;
                    }
            }
            store_block(a, j, 3 * i, G, Gi, cplx);
        }
    }
}

// Bucket assembly for graph replay: points padded to n_cap, the real count
// read from device memory; entries with i or j >= n_real form an identity block.
// A batch of systems of one bucket is one launch: system z = blockIdx.z has its
// points at + 3 z n_cap, blob widths at + z n_cap, real count at + z, and its
// matrix at out + z sys_stride.
__device__ __forceinline__ void bucket_system(AsmArgs &a, const int64_t *&n_real_p) {
    const int64_t z = blockIdx.z;
    a.tg += 3 * z * a.M;
    a.src += 3 * z * a.N;
    a.eps += z * a.N;
    a.out = (char *)a.out + z * a.sys_stride * (a.out_type == FLG_F64 ? 8 : 4);
    n_real_p += z;
}

template <int KIND>
__global__ void __launch_bounds__(128) assemble_bucket_kernel(AsmArgs a, const int64_t *n_real_p) {
    bucket_system(a, n_real_p);
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.N) return;
    const int64_t nr = *n_real_p;
    const bool jr = j < nr;
    double sx = 0, sy = 0, sz = 0, e2 = 0;
    if (jr) {
        sx = a.src[3 * j];
        sy = a.src[3 * j + 1];
        sz = a.src[3 * j + 2];
        const double e = a.eps[j];
        e2 = e * e;
    }
    for (int64_t i = blockIdx.y; i < a.M; i += gridDim.y) {
        double G[9], Gi[9];
        if (jr && i < nr) {
            block_f64<KIND, false>(a.tg[3 * i], a.tg[3 * i + 1], a.tg[3 * i + 2], sx, sy, sz, e2, a.are, a.aim, G, Gi);
            store_block(a, i, 3 * j, G, Gi, false);
        } else {
            for (int q = 0; q < 9; q++) G[q] = (i == j && (q == 0 || q == 4 || q == 8)) ? 1.0 : 0.0;
            AsmArgs b = a;
            b.scale = 1.0;
            b.imu_re = 1.0;
            b.imu_im = 0.0;
            store_block(b, i, 3 * j, G, G, false);
        }
    }
}

// The same with one blob width for every point (eps[0], read from device memory at replay):
// the symmetric assembly of assemble_sym_kernel (pairs i <= j, the mirror written as is, or
// transposed for the wall kernel by reciprocity) with the bucket's identity padding.
template <int KIND, bool TRANSPOSE>
__global__ void __launch_bounds__(128) assemble_bucket_sym_kernel(AsmArgs a, const int64_t *n_real_p) {
    bucket_system(a, n_real_p);
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= a.N) return;
    const int64_t nr = *n_real_p;
    const bool jr = j < nr;
    const double e = a.eps[0], e2 = e * e;
    double sx = 0, sy = 0, sz = 0;
    if (jr) {
        sx = a.src[3 * j];
        sy = a.src[3 * j + 1];
        sz = a.src[3 * j + 2];
    }
    AsmArgs id = a;  // identity / zero blocks of the padding: unscaled
    id.scale = 1.0;
    id.imu_re = 1.0;
    id.imu_im = 0.0;
    for (int64_t i0 = (int64_t)blockIdx.y * kSymTile; i0 <= j; i0 += (int64_t)gridDim.y * kSymTile) {
        for (int t = 0; t < kSymTile; t++) {
            const int64_t i = i0 + t;
            if (i > j) break;
            double G[9], Gi[9];
            if (jr) {  // i <= j < nr: a real pair
                block_f64<KIND, false>(a.src[3 * i], a.src[3 * i + 1], a.src[3 * i + 2], sx, sy, sz, e2, a.are,
                                       a.aim, G, Gi);
                store_block(a, i, 3 * j, G, Gi, false);
                if (i == j) continue;
                if (TRANSPOSE) {
#pragma unroll
                    for (int r = 0; r < 3; r++)
#pragma unroll
                        for (int c = r + 1; c < 3; c++) {
                            const double u = G[3 * r + c];
                            G[3 * r + c] = G[3 * c + r];
                            G[3 * c + r] = u;
                        }
                }
                store_block(a, j, 3 * i, G, Gi, false);
            } else {
                for (int q = 0; q < 9; q++) G[q] = (i == j && (q == 0 || q == 4 || q == 8)) ? 1.0 : 0.0;
                store_block(id, i, 3 * j, G, G, false);
                if (i != j) store_block(id, j, 3 * i, G, G, false);
            }
        }
    }
}

// nearest-neighbour assembly: thread per (target i, force group j), members of
// group j (ascending quadrature index) summed in FP64
struct NearestArgs {
    AsmArgs a;
    const int *grp_off;   // [n_force + 1]
    const int *grp_idx;   // [Q] quadrature indices grouped by nearest
};

template <int KIND, bool CK>
__global__ void __launch_bounds__(128) assemble_nearest_kernel(NearestArgs na) {
    const AsmArgs &a = na.a;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // force point
    if (j >= a.N) return;
    const int b = na.grp_off[j], e = na.grp_off[j + 1];
    const bool cplx = CK || a.imu_im != 0.0;
    for (int64_t i = blockIdx.y; i < a.M; i += gridDim.y) {
        const double tx = a.tg[3 * i], ty = a.tg[3 * i + 1], tz = a.tg[3 * i + 2];
        double G[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, Gi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int m = b; m < e; m++) {
            const int k = na.grp_idx[m];
            const double ek = a.eps[k];
            double g[9], gi[9];
            block_f64<KIND, CK>(tx, ty, tz, a.src[3 * k], a.src[3 * k + 1], a.src[3 * k + 2], ek * ek, a.are, a.aim,
                                g, gi);
            for (int q = 0; q < 9; q++) {
                G[q] += g[q];
                Gi[q] += gi[q];
            }
        }
        store_block(a, i, 3 * j, G, Gi, cplx);
    }
}

// ---- grouping of quadrature points by nearest force point -------------------
__global__ void group_count_kernel(const int64_t *nearest, int64_t Q, int64_t nf, int *counts, int *bad) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Q) return;
    const int64_t j = nearest[k];
    if (j < 0 || j >= nf) {
        atomicExch(bad, 1);
        return;
    }
    atomicAdd(&counts[j], 1);
}

// single-block exclusive scan of n ints (loops over 1024-element chunks)
__global__ void scan_small_kernel(const int *in, int *out, int64_t n) {
    __shared__ int sm[1024];
    __shared__ int carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < n; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const int v = i < n ? in[i] : 0;
        sm[threadIdx.x] = v;
        __syncthreads();
        for (int w = 1; w < 1024; w <<= 1) {
            int t = (int)threadIdx.x >= w ? sm[threadIdx.x - w] : 0;
            __syncthreads();
            sm[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < n) out[i] = carry + sm[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sm[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[n] = carry;
}

__global__ void group_scatter_kernel(const int64_t *nearest, int64_t Q, int64_t nf, const int *off, int *cursor,
                                     int *idx) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Q) return;
    const int64_t j = nearest[k];
    if (j < 0 || j >= nf) return;
    idx[off[j] + atomicAdd(&cursor[j], 1)] = (int)k;
}

__global__ void group_sort_kernel(const int *off, int64_t nf, int *idx) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nf) return;
    const int b = off[j], e = off[j + 1];
    for (int k = b + 1; k < e; k++) {
        int v = idx[k], m = k - 1;
        while (m >= b && idx[m] > v) {
            idx[m + 1] = idx[m];
            m--;
        }
        idx[m + 1] = v;
    }
}

// ---- swimmer rows / columns (swimming.py:90-99) ------------------------------
struct SwimArgs {
    const double *x;
    int64_t N;
    double x0[3];
    const double *x0_dev;  // when set, the origin is read from device memory (graph replays)
    const double *X;
    const int64_t *nearest;
    int64_t Q;
    void *A;
    int out_type;
    int64_t ld;
};

__device__ __forceinline__ void put(const SwimArgs &s, int64_t r, int64_t c, double v) {
    if (s.out_type == FLG_F64) ((double *)s.A)[r * s.ld + c] = v;
    else ((float *)s.A)[r * s.ld + c] = (float)v;
}

// thread per force point m: its 3 rows of the [-I | r x] columns, and its
// 3 columns of the net-force / net-torque rows
__global__ void swimmer_kernel(SwimArgs s) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n3 = 3 * s.N;
    if (m < s.N) {
        const double o0 = s.x0_dev ? s.x0_dev[0] : s.x0[0], o1 = s.x0_dev ? s.x0_dev[1] : s.x0[1],
                     o2 = s.x0_dev ? s.x0_dev[2] : s.x0[2];
        const double r0 = s.x[3 * m] - o0, r1 = s.x[3 * m + 1] - o1, r2 = s.x[3 * m + 2] - o2;
        // cross matrix C(v): C @ w = v x w  (swimming.py:33-40)
        const double C[9] = {0.0, -r2, r1, r2, 0.0, -r0, -r1, r0, 0.0};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                put(s, 3 * m + a, n3 + b, a == b ? -1.0 : 0.0);
                put(s, 3 * m + a, n3 + 3 + b, C[3 * a + b]);
            }
        // count and sum of the quadrature points of group m, ascending k
        double cnt = 0.0, X0 = 0.0, X1 = 0.0, X2 = 0.0;
        for (int64_t k = 0; k < s.Q; k++)
            if (s.nearest[k] == m) {
                cnt += 1.0;
                X0 += s.X[3 * k];
                X1 += s.X[3 * k + 1];
                X2 += s.X[3 * k + 2];
            }
        const double D[9] = {0.0, -X2, X1, X2, 0.0, -X0, -X1, X0, 0.0};
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                put(s, n3 + a, 3 * m + b, a == b ? cnt : 0.0);
                put(s, n3 + 3 + a, 3 * m + b, D[3 * a + b]);
            }
    }
    if (m < 36) put(s, n3 + m / 6, n3 + m % 6, 0.0);
}

// ---- FP64 GEMV (row-major): warp per row ------------------------------------
__global__ void __launch_bounds__(256) gemv_f64_kernel(int64_t nr, int64_t nc, const double *A, int64_t ld,
                                                       const double *x, double *y) {
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= nr) return;
    const double *a = A + row * ld;
    double acc = 0.0;
    if ((ld % 2 == 0) && (((uintptr_t)A & 15) == 0) && (((uintptr_t)x & 15) == 0)) {
        const double2 *a2 = (const double2 *)a;
        const double2 *x2 = (const double2 *)x;
        const int64_t nc2 = nc / 2;
        int64_t c = lane;
        // four independent 16-byte loads in flight per lane
        for (; c + 96 < nc2; c += 128) {
            double2 av[4], xv[4];
#pragma unroll
            for (int u = 0; u < 4; u++) av[u] = __ldcs(a2 + c + 32 * u), xv[u] = x2[c + 32 * u];
#pragma unroll
            for (int u = 0; u < 4; u++) acc = fma(av[u].y, xv[u].y, fma(av[u].x, xv[u].x, acc));
        }
        for (; c < nc2; c += 32) {
            const double2 av = __ldcs(a2 + c), xv = x2[c];
            acc = fma(av.x, xv.x, acc);
            acc = fma(av.y, xv.y, acc);
        }
        if ((nc & 1) && lane == 0) acc = fma(a[nc - 1], x[nc - 1], acc);
    } else {
        for (int64_t c = lane; c < nc; c += 32) acc = fma(a[c], x[c], acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[row] = acc;
}

// y (FP64) = A (FP32, row-major) x (FP64): the inner matvec of GMRES-IR.  The
// product is formed to near-FP64 accuracy in FP32 arithmetic, so that GB300's
// narrow FP64 pipe stays out of the loop: x = xh + xl (two FP32 parts), each
// a xh exactly as p + pe (TwoProd by FMA), the running sum s by TwoSum with its
// rounding errors, pe and a xl collected in a compensation c (Ogita, Rump and
// Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005).  The
// _rn intrinsics keep the compiler from contracting the error-free steps.  A
// warp per two rows, 32 rows per block; x goes through shared memory in chunks.
// columns of x staged in shared memory per pass (48 KB for the split x: the static limit)
#ifndef FLG_GV_CHUNK
#define FLG_GV_CHUNK 6144
#endif
constexpr int kGvWarps = 16, kGvRpw = 2, kGvRows = kGvWarps * kGvRpw, kGvChunk = FLG_GV_CHUNK;

__device__ __forceinline__ void dot2_step(float &s, float &c, float a, float xh, float xl) {
    const float p = __fmul_rn(a, xh);
    const float pe = fmaf(a, xh, -p);
    const float t = __fadd_rn(s, p);
    const float z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(p, z));
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, fmaf(a, xl, pe)));
}

// SPLIT: x arrives already split into FP32 parts xh_g, xl_g (global); otherwise each
// block splits its chunk of the FP64 x.  The loads of the next iteration are issued
// before the Dot2 chains of the current one.
template <bool SPLIT>
__global__ void __launch_bounds__(512) gemv_f32_kernel(int64_t nr, int64_t nc, const float *A, int64_t ld,
                                                       const double *x, const float *xh_g, const float *xl_g,
                                                       double *y) {
    __shared__ __align__(16) float xh[kGvChunk], xl[kGvChunk];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t row0 = (int64_t)blockIdx.x * kGvRows + warp * kGvRpw;
    const bool vec = (ld % 4 == 0) && (((uintptr_t)A & 15) == 0);
    float s[kGvRpw][4], c[kGvRpw][4];
#pragma unroll
    for (int rr = 0; rr < kGvRpw; rr++)
#pragma unroll
        for (int u = 0; u < 4; u++) s[rr][u] = 0.0f, c[rr][u] = 0.0f;
    // rows past the end read row 0 (their sums are discarded)
    const float *arow[kGvRpw];
#pragma unroll
    for (int rr = 0; rr < kGvRpw; rr++) arow[rr] = A + (row0 + rr < nr ? row0 + rr : 0) * ld;
    for (int64_t c0 = 0; c0 < nc; c0 += kGvChunk) {
        const int cw = (int)min((int64_t)kGvChunk, nc - c0);
        __syncthreads();
        if (SPLIT) {
            for (int k = threadIdx.x; k < cw; k += blockDim.x) {
                xh[k] = xh_g[c0 + k];
                xl[k] = xl_g[c0 + k];
            }
        } else {
            for (int k = threadIdx.x; k < cw; k += blockDim.x) {
                const double v = x[c0 + k];
                const float h = __double2float_rn(v);
                xh[k] = h;
                xl[k] = __double2float_rn(v - (double)h);
            }
        }
        __syncthreads();
        if (row0 >= nr) continue;
        if (vec && cw % 4 == 0) {
            const float4 *h4 = reinterpret_cast<const float4 *>(xh);
            const float4 *l4 = reinterpret_cast<const float4 *>(xl);
            const int n4 = cw / 4;
            const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
            float4 v[kGvRpw], nv[kGvRpw];
            int k = lane;
#pragma unroll
            for (int rr = 0; rr < kGvRpw; rr++)
                v[rr] = k < n4 ? __ldcs(reinterpret_cast<const float4 *>(arow[rr] + c0) + k) : z4;
            for (; k < n4; k += 32) {
                const int kn = k + 32;
#pragma unroll
                for (int rr = 0; rr < kGvRpw; rr++)
                    nv[rr] = kn < n4 ? __ldcs(reinterpret_cast<const float4 *>(arow[rr] + c0) + kn) : z4;
                const float4 h = h4[k], l = l4[k];
#pragma unroll
                for (int rr = 0; rr < kGvRpw; rr++) {
                    dot2_step(s[rr][0], c[rr][0], v[rr].x, h.x, l.x);
                    dot2_step(s[rr][1], c[rr][1], v[rr].y, h.y, l.y);
                    dot2_step(s[rr][2], c[rr][2], v[rr].z, h.z, l.z);
                    dot2_step(s[rr][3], c[rr][3], v[rr].w, h.w, l.w);
                    v[rr] = nv[rr];
                }
            }
        } else {
            for (int k = lane; k < cw; k += 32) {
#pragma unroll
                for (int rr = 0; rr < kGvRpw; rr++) dot2_step(s[rr][0], c[rr][0], arow[rr][c0 + k], xh[k], xl[k]);
            }
        }
    }
#pragma unroll
    for (int rr = 0; rr < kGvRpw; rr++) {
        double acc = 0.0;
#pragma unroll
        for (int u = 0; u < 4; u++) acc += (double)s[rr][u] + (double)c[rr][u];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0 && row0 + rr < nr) y[row0 + rr] = acc;
    }
}

// x (FP64) -> xh + xl (FP32 parts, exactly xh + xl = x up to 2^-48 relative)
__global__ void split_f64_kernel(const double *x, float *xh, float *xl, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    const float h = __double2float_rn(v);
    xh[i] = h;
    xl[i] = __double2float_rn(v - (double)h);
}

__global__ void convert_f64_f32_kernel(int64_t nr, int64_t nc, const double *src, int64_t lds, float *dst,
                                       int64_t ldd) {
    const int64_t r = blockIdx.y;
    for (int64_t rr = r; rr < nr; rr += gridDim.y)
        for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += (int64_t)gridDim.x * blockDim.x)
            dst[rr * ldd + c] = (float)src[rr * lds + c];
}

// dst1 = dst2 = (float) src, read once: the mixed solve's two FP32 copies of the FP64 matrix
// (the one factored in place and the one of the inner matvecs).  Each thread converts four
// consecutive elements of a row (independent loads in flight); dst2 may be null.
__global__ void __launch_bounds__(256) convert2_f64_f32_kernel(int64_t nr, int64_t nc, const double *src,
                                                              int64_t lds, float *dst1, float *dst2, int64_t ldd) {
    const int64_t per_row = (nc + 3) / 4;
    const int64_t total = nr * per_row;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = q / per_row, c0 = (q - r * per_row) * 4;
        const double *s = src + r * lds + c0;
        float v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) v[k] = c0 + k < nc ? (float)s[k] : 0.0f;
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (c0 + k < nc) {
                dst1[r * ldd + c0 + k] = v[k];
                if (dst2) dst2[r * ldd + c0 + k] = v[k];
            }
    }
}

// ---- host side ----------------------------------------------------------------
static int prepare(int kind, double are, double aim, double mu_re, double mu_im, int out_type, AsmArgs &a) {
    FLG_TRY(check_kernel_args(kind, are, aim));
    FLG_REQUIRE(!(mu_re == 0.0 && mu_im == 0.0), "mu must be non-zero");
    FLG_REQUIRE(out_type >= FLG_F64 && out_type <= FLG_BF16, "unknown out_type %d", out_type);
    const bool cplx = (kind == FLG_BRINKMANLET && aim != 0.0) || mu_im != 0.0;
    FLG_REQUIRE(!cplx || out_type == FLG_C128, "a complex kernel or viscosity needs out_type FLG_C128");
    a.are = are;
    a.aim = aim;
    a.scale = kind == FLG_BRINKMANLET ? 1.0 / (4.0 * kPi) : 1.0 / (8.0 * kPi);
    const double d = mu_re * mu_re + mu_im * mu_im;
    a.imu_re = mu_im == 0.0 ? 1.0 / mu_re : mu_re / d;
    a.imu_im = mu_im == 0.0 ? 0.0 : -mu_im / d;
    a.out_type = out_type;
    return FLG_OK;
}

template <template <int, bool> class Launch, typename Arg>
static void dispatch(int kind, bool ck, dim3 grid, int threads, cudaStream_t st, const Arg &arg) {
    if (kind == FLG_STOKESLET) Launch<FLG_STOKESLET, false>::go(grid, threads, st, arg);
    else if (kind == FLG_WALL) Launch<FLG_WALL, false>::go(grid, threads, st, arg);
    else if (ck) Launch<FLG_BRINKMANLET, true>::go(grid, threads, st, arg);
    else Launch<FLG_BRINKMANLET, false>::go(grid, threads, st, arg);
}

template <int K, bool C>
struct LaunchAsm {
    static void go(dim3 g, int t, cudaStream_t st, const AsmArgs &a) { assemble_kernel<K, C><<<g, t, 0, st>>>(a); }
};
template <int K, bool C>
struct LaunchNearest {
    static void go(dim3 g, int t, cudaStream_t st, const NearestArgs &a) {
        assemble_nearest_kernel<K, C><<<g, t, 0, st>>>(a);
    }
};

static dim3 asm_grid(int64_t M, int64_t N) {
    return dim3((unsigned)ceil_div(N, 128), (unsigned)std::min<int64_t>(M, 65535));
}

}  // namespace flg

using namespace flg;

extern "C" int flg_assemble(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                            const double *sources, const double *eps, int64_t N, double mu_re, double mu_im,
                            void *out, int out_type, int64_t ld, void *stream) {
    FLG_RANGE("flg_assemble");
    AsmArgs a{};
    FLG_TRY(prepare(kind, alpha_re, alpha_im, mu_re, mu_im, out_type, a));
    FLG_REQUIRE(M >= 0 && N >= 0, "negative sizes");
    FLG_REQUIRE(ld >= 3 * N, "ld (%lld) < 3N (%lld)", (long long)ld, (long long)(3 * N));
    if (M == 0 || N == 0) return FLG_OK;
    FLG_REQUIRE(targets && sources && eps && out, "null pointer");
    a.tg = targets;
    a.M = M;
    a.src = sources;
    a.eps = eps;
    a.N = N;
    a.out = out;
    a.ld = ld;
    cudaStream_t st = as_stream(stream);
    prof_begin(FLG_SLOT_ASSEMBLE, st);
    dispatch<LaunchAsm>(kind, kind == FLG_BRINKMANLET && alpha_im != 0.0, asm_grid(M, N), 128, st, a);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_ASSEMBLE, st);
    return FLG_OK;
}

extern "C" int flg_assemble_self_uniform(int kind, double alpha_re, double alpha_im, const double *points, int64_t N,
                                         double eps, double mu_re, double mu_im, void *out, int out_type, int64_t ld,
                                         void *stream) {
    FLG_RANGE("flg_assemble_self_uniform");
    AsmArgs a{};
    FLG_TRY(prepare(kind, alpha_re, alpha_im, mu_re, mu_im, out_type, a));
    FLG_REQUIRE(N >= 0, "negative size");
    FLG_REQUIRE(ld >= 3 * N, "ld (%lld) < 3N (%lld)", (long long)ld, (long long)(3 * N));
    if (N == 0) return FLG_OK;
    FLG_REQUIRE(points && out, "null pointer");
    a.tg = points;
    a.M = N;
    a.src = points;
    a.eps = nullptr;
    a.N = N;
    a.out = out;
    a.ld = ld;
    cudaStream_t st = as_stream(stream);
    const dim3 grid((unsigned)ceil_div(N, 128), (unsigned)std::min<int64_t>(ceil_div(N, kSymTile), 65535));
    const double e2 = eps * eps;
    prof_begin(FLG_SLOT_ASSEMBLE, st);
    if (kind == FLG_STOKESLET) assemble_sym_kernel<FLG_STOKESLET, false, false><<<grid, 128, 0, st>>>(a, e2);
    else if (kind == FLG_WALL) assemble_sym_kernel<FLG_WALL, false, true><<<grid, 128, 0, st>>>(a, e2);
    else if (alpha_im != 0.0) assemble_sym_kernel<FLG_BRINKMANLET, true, false><<<grid, 128, 0, st>>>(a, e2);
    else assemble_sym_kernel<FLG_BRINKMANLET, false, false><<<grid, 128, 0, st>>>(a, e2);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_ASSEMBLE, st);
    return FLG_OK;
}

// nbat systems of one bucket (bucket_system), the symmetric form when every point of a
// system has the blob width eps[0] of that system
static int assemble_bucket_batch(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                                 bool uniform, const int64_t *n_real, int64_t n_cap, int nbat, double mu_re,
                                 void *out, int out_type, int64_t ld, int64_t stride_out, cudaStream_t st) {
    AsmArgs a{};
    FLG_TRY(prepare(kind, alpha_re, alpha_im, mu_re, 0.0, out_type, a));
    FLG_REQUIRE(!(kind == FLG_BRINKMANLET && alpha_im != 0.0), "bucket assembly is real only");
    FLG_REQUIRE(out_type == FLG_F64 || out_type == FLG_F32, "bucket assembly writes FLG_F64 or FLG_F32");
    FLG_REQUIRE(n_cap >= 0 && ld >= 3 * n_cap, "bad bucket shape");
    FLG_REQUIRE(nbat >= 1 && nbat <= 65535 && (nbat == 1 || stride_out >= 3 * n_cap * ld), "bad bucket batch");
    if (n_cap == 0) return FLG_OK;
    FLG_REQUIRE(points && eps && n_real && out, "null pointer");
    a.tg = points;
    a.M = n_cap;
    a.src = points;
    a.eps = eps;
    a.N = n_cap;
    a.out = out;
    a.ld = ld;
    a.sys_stride = stride_out;
    prof_begin(FLG_SLOT_ASSEMBLE, st);
    if (uniform) {
        const dim3 grid((unsigned)ceil_div(n_cap, 128), (unsigned)std::min<int64_t>(ceil_div(n_cap, kSymTile), 65535),
                        (unsigned)nbat);
        if (kind == FLG_STOKESLET) assemble_bucket_sym_kernel<FLG_STOKESLET, false><<<grid, 128, 0, st>>>(a, n_real);
        else if (kind == FLG_WALL) assemble_bucket_sym_kernel<FLG_WALL, true><<<grid, 128, 0, st>>>(a, n_real);
        else assemble_bucket_sym_kernel<FLG_BRINKMANLET, false><<<grid, 128, 0, st>>>(a, n_real);
    } else {
        dim3 grid = asm_grid(n_cap, n_cap);
        grid.z = (unsigned)nbat;
        if (kind == FLG_STOKESLET) assemble_bucket_kernel<FLG_STOKESLET><<<grid, 128, 0, st>>>(a, n_real);
        else if (kind == FLG_WALL) assemble_bucket_kernel<FLG_WALL><<<grid, 128, 0, st>>>(a, n_real);
        else assemble_bucket_kernel<FLG_BRINKMANLET><<<grid, 128, 0, st>>>(a, n_real);
    }
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_ASSEMBLE, st);
    return FLG_OK;
}

extern "C" int flg_assemble_bucket_uniform(int kind, double alpha_re, double alpha_im, const double *points,
                                           const double *eps, const int64_t *n_real, int64_t n_cap, double mu_re,
                                           void *out, int out_type, int64_t ld, void *stream) {
    FLG_RANGE("flg_assemble_bucket_uniform");
    return assemble_bucket_batch(kind, alpha_re, alpha_im, points, eps, true, n_real, n_cap, 1, mu_re, out, out_type,
                                 ld, 0, as_stream(stream));
}

extern "C" int flg_assemble_bucket(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                                   const int64_t *n_real, int64_t n_cap, double mu_re, void *out, int out_type,
                                   int64_t ld, void *stream) {
    FLG_RANGE("flg_assemble_bucket");
    return assemble_bucket_batch(kind, alpha_re, alpha_im, points, eps, false, n_real, n_cap, 1, mu_re, out, out_type,
                                 ld, 0, as_stream(stream));
}

extern "C" int flg_assemble_bucket_batched(int kind, double alpha_re, double alpha_im, const double *points,
                                           const double *eps, int uniform_eps, const int64_t *n_real, int64_t n_cap,
                                           int nbat, double mu_re, void *out, int out_type, int64_t ld,
                                           int64_t stride_out, void *stream) {
    FLG_RANGE("flg_assemble_bucket_batched");
    return assemble_bucket_batch(kind, alpha_re, alpha_im, points, eps, uniform_eps != 0, n_real, n_cap, nbat, mu_re,
                                 out, out_type, ld, stride_out, as_stream(stream));
}

extern "C" size_t flg_assemble_nearest_workspace(int64_t Q, int64_t n_force) {
    CountingArena c;
    c.take<int>(n_force + 1);  // counts / cursor
    c.take<int>(n_force + 1);  // offsets
    c.take<int>(Q + 1);        // grouped indices
    c.take<int>(1);            // bad-index flag
    return c.bytes();
}

// bad_flag: null -> check the indices and synchronize (flg_assemble_nearest); else the
// device int receives 1 if an index lies outside [0, n_force) and nothing waits
// (out-of-range indices are skipped by every kernel, so the launch sequence is safe)
static int assemble_nearest_impl(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                                 const double *quad, const int64_t *nearest, const double *eps, int64_t Q,
                                 int64_t n_force, double mu_re, double mu_im, void *out, int out_type, int64_t ld,
                                 void *work, size_t work_bytes, void *stream, int *bad_flag) {
    AsmArgs a{};
    FLG_TRY(prepare(kind, alpha_re, alpha_im, mu_re, mu_im, out_type, a));
    FLG_REQUIRE(out_type != FLG_BF16, "assemble_nearest writes FLG_F64, FLG_C128 or FLG_F32");
    FLG_REQUIRE(M >= 0 && Q >= 0 && n_force >= 0, "negative sizes");
    FLG_REQUIRE(Q < (1LL << 31) && n_force < (1LL << 31), "at most 2^31 - 1 quadrature / force points");
    FLG_REQUIRE(ld >= 3 * n_force, "ld < 3 n_force");
    if (M == 0 || n_force == 0) return FLG_OK;
    FLG_REQUIRE(targets && out && (Q == 0 || (quad && nearest && eps)), "null pointer");
    Arena ar(work, work_bytes);
    int *counts = ar.take<int>(n_force + 1);
    int *off = ar.take<int>(n_force + 1);
    int *idx = ar.take<int>(Q + 1);
    int *bad = ar.take<int>(1);
    FLG_REQUIRE(counts && off && idx && bad, "workspace too small (%zu bytes)", work_bytes);
    if (bad_flag) bad = bad_flag;
    cudaStream_t st = as_stream(stream);
    FLG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (n_force + 1), st));
    FLG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), st));
    if (Q > 0) {
        group_count_kernel<<<(unsigned)ceil_div(Q, 256), 256, 0, st>>>(nearest, Q, n_force, counts, bad);
        FLG_LAUNCH_CHECK();
    }
    scan_small_kernel<<<1, 1024, 0, st>>>(counts, off, n_force);
    FLG_LAUNCH_CHECK();
    FLG_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (n_force + 1), st));
    if (Q > 0) {
        group_scatter_kernel<<<(unsigned)ceil_div(Q, 256), 256, 0, st>>>(nearest, Q, n_force, off, counts, idx);
        FLG_LAUNCH_CHECK();
        group_sort_kernel<<<(unsigned)ceil_div(n_force, 256), 256, 0, st>>>(off, n_force, idx);
        FLG_LAUNCH_CHECK();
    }
    a.tg = targets;
    a.M = M;
    a.src = quad;
    a.eps = eps;
    a.N = n_force;
    a.out = out;
    a.ld = ld;
    NearestArgs na{a, off, idx};
    prof_begin(FLG_SLOT_ASSEMBLE, st);
    dispatch<LaunchNearest>(kind, kind == FLG_BRINKMANLET && alpha_im != 0.0, asm_grid(M, n_force), 128, st, na);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_ASSEMBLE, st);
    if (bad_flag) return FLG_OK;
    int hbad = 0;
    FLG_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    FLG_REQUIRE(hbad == 0, "nearest indices must lie in [0, n_force)");
    return FLG_OK;
}

extern "C" int flg_assemble_nearest(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                                    const double *quad, const int64_t *nearest, const double *eps, int64_t Q,
                                    int64_t n_force, double mu_re, double mu_im, void *out, int out_type, int64_t ld,
                                    void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_assemble_nearest");
    return assemble_nearest_impl(kind, alpha_re, alpha_im, targets, M, quad, nearest, eps, Q, n_force, mu_re, mu_im,
                                 out, out_type, ld, work, work_bytes, stream, nullptr);
}

extern "C" int flg_assemble_nearest_async(int kind, double alpha_re, double alpha_im, const double *targets,
                                          int64_t M, const double *quad, const int64_t *nearest, const double *eps,
                                          int64_t Q, int64_t n_force, double mu_re, double mu_im, void *out,
                                          int out_type, int64_t ld, int *bad_flag, void *work, size_t work_bytes,
                                          void *stream) {
    FLG_REQUIRE(bad_flag, "null flag");
    return assemble_nearest_impl(kind, alpha_re, alpha_im, targets, M, quad, nearest, eps, Q, n_force, mu_re, mu_im,
                                 out, out_type, ld, work, work_bytes, stream, bad_flag);
}

extern "C" int flg_swimmer_constraints(const double *x, int64_t N, const double *x0_host, const double *X,
                                       const int64_t *nearest, int64_t Q, void *A, int out_type, int64_t ld,
                                       void *stream) {
    FLG_RANGE("flg_swimmer_constraints");
    FLG_REQUIRE(N >= 0 && Q >= 0, "negative sizes");
    FLG_REQUIRE(out_type == FLG_F64 || out_type == FLG_F32, "swimmer system is FLG_F64 or FLG_F32");
    FLG_REQUIRE(ld >= 3 * N + 6, "ld < 3N + 6");
    FLG_REQUIRE(x0_host && A && (N == 0 || x) && (Q == 0 || (X && nearest)), "null pointer");
    SwimArgs s{x, N, {x0_host[0], x0_host[1], x0_host[2]}, nullptr, X, nearest, Q, A, out_type, ld};
    const int64_t threads = std::max<int64_t>(N, 36);
    swimmer_kernel<<<(unsigned)ceil_div(threads, 128), 128, 0, as_stream(stream)>>>(s);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_swimmer_constraints_dev(const double *x, int64_t N, const double *x0_dev, const double *X,
                                           const int64_t *nearest, int64_t Q, void *A, int out_type, int64_t ld,
                                           void *stream) {
    FLG_REQUIRE(N >= 0 && Q >= 0, "negative sizes");
    FLG_REQUIRE(out_type == FLG_F64 || out_type == FLG_F32, "swimmer system is FLG_F64 or FLG_F32");
    FLG_REQUIRE(ld >= 3 * N + 6, "ld < 3N + 6");
    FLG_REQUIRE(x0_dev && A && (N == 0 || x) && (Q == 0 || (X && nearest)), "null pointer");
    SwimArgs s{x, N, {0.0, 0.0, 0.0}, x0_dev, X, nearest, Q, A, out_type, ld};
    const int64_t threads = std::max<int64_t>(N, 36);
    swimmer_kernel<<<(unsigned)ceil_div(threads, 128), 128, 0, as_stream(stream)>>>(s);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_gemv_f64(int64_t n_rows, int64_t n_cols, const double *A, int64_t ld, const double *x, double *y,
                            void *stream) {
    FLG_REQUIRE(n_rows >= 0 && n_cols >= 0 && ld >= n_cols, "bad GEMV shape");
    if (n_rows == 0) return FLG_OK;
    cudaStream_t st = as_stream(stream);
    prof_begin(FLG_SLOT_GEMV, st);
    gemv_f64_kernel<<<(unsigned)ceil_div(n_rows * 32, 256), 256, 0, st>>>(n_rows, n_cols, A, ld, x, y);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_GEMV, st);
    return FLG_OK;
}

extern "C" int flg_gemv_f32(int64_t n_rows, int64_t n_cols, const float *A, int64_t ld, const double *x, double *y,
                            void *stream) {
    FLG_REQUIRE(n_rows >= 0 && n_cols >= 0 && ld >= n_cols, "bad GEMV shape");
    if (n_rows == 0) return FLG_OK;
    cudaStream_t st = as_stream(stream);
    prof_begin(FLG_SLOT_GEMV, st);
    gemv_f32_kernel<false><<<(unsigned)ceil_div(n_rows, kGvRows), 32 * kGvWarps, 0, st>>>(n_rows, n_cols, A, ld, x,
                                                                                         nullptr, nullptr, y);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_GEMV, st);
    return FLG_OK;
}

namespace flg {
// the same product with x split once into xsplit[0, n_cols) (high parts) and
// xsplit[n_cols, 2 n_cols) (low parts), a caller workspace (GMRES-IR)
int gemv_f32_presplit(int64_t n_rows, int64_t n_cols, const float *A, int64_t ld, const double *x, float *xsplit,
                      double *y, cudaStream_t st) {
    FLG_REQUIRE(n_rows >= 0 && n_cols >= 0 && ld >= n_cols, "bad GEMV shape");
    if (n_rows == 0) return FLG_OK;
    if (n_cols > 0) {
        split_f64_kernel<<<(unsigned)ceil_div(n_cols, 256), 256, 0, st>>>(x, xsplit, xsplit + n_cols, n_cols);
        FLG_LAUNCH_CHECK();
    }
    prof_begin(FLG_SLOT_GEMV, st);
    gemv_f32_kernel<true><<<(unsigned)ceil_div(n_rows, kGvRows), 32 * kGvWarps, 0, st>>>(
        n_rows, n_cols, A, ld, nullptr, xsplit, xsplit + n_cols, y);
    FLG_LAUNCH_CHECK();
    prof_end(FLG_SLOT_GEMV, st);
    return FLG_OK;
}
}  // namespace flg

// nearest force point of every quadrature point (the reference's k-d tree query,
// core/assemble.py:61-65): exhaustive, FP64 squared distances, the first index
// on ties; force points staged through shared memory in tiles of kNnTile
constexpr int kNnTile = 1024;
__global__ void __launch_bounds__(256) nearest_kernel(const double *quad, int64_t Q, const double *force, int64_t N,
                                                      int64_t *out) {
    __shared__ double fx[kNnTile], fy[kNnTile], fz[kNnTile];
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    double px = 0.0, py = 0.0, pz = 0.0;
    if (q < Q) px = quad[3 * q], py = quad[3 * q + 1], pz = quad[3 * q + 2];
    double best = INFINITY;
    int64_t bi = 0;
    for (int64_t t0 = 0; t0 < N; t0 += kNnTile) {
        const int nt = (int)min((int64_t)kNnTile, N - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < nt; k += blockDim.x) {
            fx[k] = force[3 * (t0 + k)];
            fy[k] = force[3 * (t0 + k) + 1];
            fz[k] = force[3 * (t0 + k) + 2];
        }
        __syncthreads();
        for (int k = 0; k < nt; k++) {
            const double dx = px - fx[k], dy = py - fy[k], dz = pz - fz[k];
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < best) {
                best = d2;
                bi = t0 + k;
            }
        }
    }
    if (q < Q) out[q] = bi;
}

extern "C" int flg_nearest_neighbors(const double *quad, int64_t Q, const double *force, int64_t N, int64_t *out,
                                     void *stream) {
    FLG_RANGE("flg_nearest_neighbors");
    FLG_REQUIRE(Q >= 0 && N >= 0, "negative sizes");
    if (Q == 0) return FLG_OK;
    FLG_REQUIRE(N > 0, "no force points to search");
    FLG_REQUIRE(quad && force && out, "null pointer");
    nearest_kernel<<<(unsigned)ceil_div(Q, 256), 256, 0, as_stream(stream)>>>(quad, Q, force, N, out);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

// grid point (i, j, k) -> row i + nx (j + ny k): x fastest, then y, then z (VTK point order)
__global__ void grid_points_kernel(const double *xa, int64_t nx, const double *ya, int64_t ny, const double *za,
                                   int64_t nz, double *out) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nx * ny * nz) return;
    const int64_t i = p % nx, j = (p / nx) % ny, k = p / (nx * ny);
    out[3 * p] = xa[i];
    out[3 * p + 1] = ya[j];
    out[3 * p + 2] = za[k];
}

extern "C" int flg_grid_points(const double *x_axis, int64_t nx, const double *y_axis, int64_t ny,
                               const double *z_axis, int64_t nz, double *points, void *stream) {
    FLG_REQUIRE(nx >= 0 && ny >= 0 && nz >= 0, "negative grid size");
    const int64_t np = nx * ny * nz;
    if (np == 0) return FLG_OK;
    FLG_REQUIRE(x_axis && y_axis && z_axis && points, "null pointer");
    grid_points_kernel<<<(unsigned)ceil_div(np, 256), 256, 0, as_stream(stream)>>>(x_axis, nx, y_axis, ny, z_axis,
                                                                                    nz, points);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_convert_f64_f32x2(int64_t n_rows, int64_t n_cols, const double *src, int64_t lds, float *dst1,
                                     float *dst2, int64_t ldd, void *stream) {
    FLG_REQUIRE(n_rows >= 0 && n_cols >= 0 && lds >= n_cols && ldd >= n_cols && dst1, "bad conversion shape");
    if (n_rows == 0 || n_cols == 0) return FLG_OK;
    const int64_t work = n_rows * ((n_cols + 3) / 4);
    const unsigned grid = (unsigned)std::min<int64_t>(ceil_div(work, 256), (int64_t)sm_count() * 16);
    convert2_f64_f32_kernel<<<grid, 256, 0, as_stream(stream)>>>(n_rows, n_cols, src, lds, dst1, dst2, ldd);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

extern "C" int flg_convert_f64_f32(int64_t n_rows, int64_t n_cols, const double *src, int64_t lds, float *dst,
                                   int64_t ldd, void *stream) {
    FLG_REQUIRE(n_rows >= 0 && n_cols >= 0 && lds >= n_cols && ldd >= n_cols, "bad conversion shape");
    if (n_rows == 0 || n_cols == 0) return FLG_OK;
    dim3 grid((unsigned)std::min<int64_t>(ceil_div(n_cols, 256), 64), (unsigned)std::min<int64_t>(n_rows, 65535));
    convert_f64_f32_kernel<<<grid, 256, 0, as_stream(stream)>>>(n_rows, n_cols, src, lds, dst, ldd);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}
