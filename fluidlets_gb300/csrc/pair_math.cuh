// pair_math.cuh -- per-pair kernel arithmetic, templated on float / double.
//
// Every kernel is applied in "vector form": the 3x3 block G(x, y) is never
// stored; its product with the strength f is accumulated directly.  The global
// scale (1/8pi for the Stokeslet and the wall kernel, 1/4pi for the
// Brinkmanlet) and the division by mu are applied once per target.
//
// Stokeslet (kernels/stokeslet3d.py:22-50):  with Q = r^2 + e^2, s = Q^-1/2
//     8 pi u = (s + e^2 s^3) f + s^3 (f.d) d        [= H1 f + H2 (f.d) d]
//
// Brinkmanlet (kernels/brinkmanlet3d.py:52-104): R = Q^1/2, z = alpha R,
//     4 pi u = (f1(z)/R + e^2 f2(z)/R^3) f + f2(z)/R^3 (f.d) d
// with the reference's 24-term Taylor series of f1, f2 below z = 0.5 and the
// closed forms above (complex alpha: |z| < 0.5, complex z).
//
// Wall Stokeslet (kernels/images.py:26-89, Ainley et al. 2008), factored.
// For a target at height t and a source at height h, with d = x - y,
// dm = t - h, dp = t + h (displacement from the image point), QF = |d|^2+e^2,
// QI = |d - (0,0,dm) + (0,0,dp)|^2 + e^2, sF = QF^-1/2, s = QI^-1/2, the free
// Stokeslet plus the image system (Stokeslet, dipole, doublet, rotlet) is
// algebraically identical to
//     8 pi u_j = 2th [ cxy f_j + d_j (Z3 (f.dF) - 3 s^5 P) ]              (j = x, y)
//     8 pi u_z = 2th [ cz f_z + dm Z3 (f.dF) - 3 s^5 P dp ]
// where  Z1 = 2 sF^2 s^2 / (sF + s),  Z3 = Z1 (sF^2 + sF s + s^2),
//        cxy = Z1 + e^2 Z3 - s^3 + 3 e^2 s^5,  cz = Z1 + e^2 Z3 - s^3 - 3 e^2 s^5,
//        f.dF = d_x f_x + d_y f_y + dm f_z,  P = dp f_z - d_x f_x - d_y f_y.
// (The identity follows from sF - s = 4th sF^2 s^2/(sF + s).)  Every term
// carries the factor t*h, so the velocity on the wall t = 0 is exactly zero
// and there is no cancellation between the free and the image terms near the
// wall: the same formula is accurate in FP32 for targets close to z = 0.
#pragma once
#include <cuda_runtime.h>

namespace flg {

// ---- fast elementary functions --------------------------------------------
// FP32: the PTX approximate instructions (MUFU), flush-to-zero.
__device__ __forceinline__ float rsq(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float expneg(float z) { return ex2(-1.4426950408889634f * z); }
// FP64: CUDA's double-precision library functions.
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ double rcp(double x) { return __drcp_rn(x); }
__device__ __forceinline__ double expneg(double z) { return exp(-z); }

template <typename T>
__device__ __forceinline__ T fmaT(T a, T b, T c) { return fma(a, b, c); }
template <>
__device__ __forceinline__ float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }
// explicitly rounded subtraction: the displacement that feeds the near/far
// predicate must be computed the same way in every kernel
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// Brinkmanlet series coefficients (kernels/brinkmanlet3d.py:46-49):
//   C1[n] = (-1)^n (1/(n+2)! - 1/(n+1)! + 1/n!)
//   C2[n] = (-1)^(n+1) (3/(n+2)! - 3/(n+1)! + 1/n!)
// evaluated at compile time in double, left to right as in the reference.
constexpr int kBrNTerms64 = 24;  // reference N_TERMS
constexpr int kBrNTerms32 = 12;  // z < 0.5: z^12/12! < 1e-12, below FP32 rounding
constexpr double br_fact(int n) {
    double f = 1.0;
    for (int k = 2; k <= n; k++) f *= (double)k;
    return f;
}
constexpr double br_c1(int n) {
    return (n % 2 ? -1.0 : 1.0) * (1.0 / br_fact(n + 2) - 1.0 / br_fact(n + 1) + 1.0 / br_fact(n));
}
constexpr double br_c2(int n) {
    return (n % 2 ? 1.0 : -1.0) * (3.0 / br_fact(n + 2) - 3.0 / br_fact(n + 1) + 1.0 / br_fact(n));
}
#define FLG_BR24(F) F(0), F(1), F(2), F(3), F(4), F(5), F(6), F(7), F(8), F(9), F(10), F(11), \
    F(12), F(13), F(14), F(15), F(16), F(17), F(18), F(19), F(20), F(21), F(22), F(23)
#define FLG_F32C1(n) (float)br_c1(n)
#define FLG_F32C2(n) (float)br_c2(n)
static __constant__ double c_br_c1[kBrNTerms64] = {FLG_BR24(br_c1)};
static __constant__ double c_br_c2[kBrNTerms64] = {FLG_BR24(br_c2)};
static __constant__ float c_br_c1f[kBrNTerms64] = {FLG_BR24(FLG_F32C1)};
static __constant__ float c_br_c2f[kBrNTerms64] = {FLG_BR24(FLG_F32C2)};

// ---- the near/far predicate ----------------------------------------------
// A pair is "near" when |d|^2 < 16 eps^2, evaluated as QF < 17 eps^2 on the
// FP32 copies of the coordinates with explicitly rounded operations, so the
// FP32 far-field kernel and the FP64 near-field kernel classify every pair
// identically.  d2 is the z displacement (t - h).
__device__ __forceinline__ float free_Q_f32(float d0, float d1, float d2, float e2) {
    return __fmaf_rn(d2, d2, __fmaf_rn(d1, d1, __fmaf_rn(d0, d0, e2)));
}

// ---- Stokeslet / Brinkmanlet: radial coefficients -------------------------
// Returns A, B with  u += A f + B (f.d) d  (before the global scale).
template <typename T>
__device__ __forceinline__ void stokeslet_AB(T s, T e2, T &A, T &B) {
    T s3 = s * s * s;
    A = fmaT(e2, s3, s);
    B = s3;
}

template <typename T, int NT>
__device__ __forceinline__ void brink_series(T z, T &f1, T &f2) {
    f1 = T(0);
    f2 = T(0);
#pragma unroll
    for (int n = NT - 1; n >= 0; n--) {
        if constexpr (sizeof(T) == 8) {
            f1 = fmaT(f1, z, T(c_br_c1[n]));
            f2 = fmaT(f2, z, T(c_br_c2[n]));
        } else {
            f1 = fmaT(f1, z, T(c_br_c1f[n]));
            f2 = fmaT(f2, z, T(c_br_c2f[n]));
        }
    }
}

// real alpha >= 0: f1 = e^-z (1 + 1/z + 1/z^2) - 1/z^2, f2 = 3/z^2 - e^-z (1 + 3/z + 3/z^2)
template <typename T>
__device__ __forceinline__ void brink_AB(T s, T Q, T e2, T alpha, T &A, T &B) {
    constexpr int NT = sizeof(T) == 8 ? kBrNTerms64 : kBrNTerms32;
    T R = Q * s;
    T z = alpha * R;
    T f1, f2;
    if (z < T(0.5)) {
        brink_series<T, NT>(z, f1, f2);
    } else {
        T E = expneg(z);
        T iz = rcp(z);
        T iz2 = iz * iz;
        f1 = fmaT(E, T(1) + iz + iz2, -iz2);
        f2 = fmaT(-E, fmaT(T(3), iz2 + iz, T(1)), T(3) * iz2);
    }
    T s3 = s * s * s;
    B = f2 * s3;
    A = fmaT(e2, B, f1 * s);
}

// complex alpha: same functions of complex z, series for |z| < 0.5
template <typename T>
struct cpx {
    T re, im;
};
template <typename T>
__device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
    return {fmaT(a.re, b.re, -a.im * b.im), fmaT(a.re, b.im, a.im * b.re)};
}

template <typename T>
__device__ __forceinline__ void brink_AB_c(T s, T Q, T e2, T are, T aim, cpx<T> &A, cpx<T> &B) {
    constexpr int NT = sizeof(T) == 8 ? kBrNTerms64 : kBrNTerms32;
    T R = Q * s;
    cpx<T> z = {are * R, aim * R};
    T az2 = z.re * z.re + z.im * z.im;
    cpx<T> f1, f2;
    if (az2 < T(0.25)) {
        f1 = {T(0), T(0)};
        f2 = {T(0), T(0)};
#pragma unroll
        for (int n = NT - 1; n >= 0; n--) {
            T c1, c2;
            if constexpr (sizeof(T) == 8) {
                c1 = c_br_c1[n];
                c2 = c_br_c2[n];
            } else {
                c1 = c_br_c1f[n];
                c2 = c_br_c2f[n];
            }
            f1 = cmul(f1, z);
            f1.re += c1;
            f2 = cmul(f2, z);
            f2.re += c2;
        }
    } else {
        // E = e^-z = e^-x (cos y - i sin y)
        T ex = expneg(z.re), sn, cs;
        if constexpr (sizeof(T) == 8) {
            sincos(z.im, &sn, &cs);
        } else {
            // range-reduce to [-pi, pi] before the approximate MUFU sin/cos
            T k = rintf(z.im * 0.15915494309189535f);
            T y = fmaf(-k, 6.283185307179586f, z.im);
            sn = __sinf(y);
            cs = __cosf(y);
        }
        cpx<T> E = {ex * cs, -ex * sn};
        T inv = rcp(az2);
        cpx<T> iz = {z.re * inv, -z.im * inv};
        cpx<T> iz2 = cmul(iz, iz);
        cpx<T> t1 = {T(1) + iz.re + iz2.re, iz.im + iz2.im};
        cpx<T> Et1 = cmul(E, t1);
        f1 = {Et1.re - iz2.re, Et1.im - iz2.im};
        cpx<T> t2 = {T(1) + T(3) * (iz.re + iz2.re), T(3) * (iz.im + iz2.im)};
        cpx<T> Et2 = cmul(E, t2);
        f2 = {T(3) * iz2.re - Et2.re, T(3) * iz2.im - Et2.im};
    }
    T s3 = s * s * s;
    B = {f2.re * s3, f2.im * s3};
    A = {fmaT(e2, B.re, f1.re * s), fmaT(e2, B.im, f1.im * s)};
}

// u += A f + B (f.d) d for one real strength vector
template <typename T>
__device__ __forceinline__ void radial_apply(T A, T B, T d0, T d1, T d2, T f0, T f1, T f2, T *u) {
    T fd = fmaT(d2, f2, fmaT(d1, f1, d0 * f0));
    T b = B * fd;
    u[0] = fmaT(A, f0, fmaT(b, d0, u[0]));
    u[1] = fmaT(A, f1, fmaT(b, d1, u[1]));
    u[2] = fmaT(A, f2, fmaT(b, d2, u[2]));
}

// ---- wall kernel, factored (see the header comment) -----------------------
template <typename T>
struct WallGeo {
    T d0, d1, dm, dp, W2, cxy, cz, Z3, s5x3;
};

// tz2 = 2 t (per target), h = source height.  MASK zeroes near pairs (QF < thr).
template <typename T, bool MASK>
__device__ __forceinline__ WallGeo<T> wall_geo(T tx, T ty, T tz, T tz2, T sx, T sy, T h, T e2, T thr) {
    WallGeo<T> g;
    g.d0 = sub_rn(tx, sx);
    g.d1 = sub_rn(ty, sy);
    g.dm = sub_rn(tz, h);
    g.dp = tz + h;
    T rq, QF;
    if constexpr (sizeof(T) == 4) {
        rq = __fmaf_rn(g.d1, g.d1, __fmaf_rn(g.d0, g.d0, e2));
        QF = __fmaf_rn(g.dm, g.dm, rq);
    } else {
        rq = fmaT(g.d1, g.d1, fmaT(g.d0, g.d0, e2));
        QF = fmaT(g.dm, g.dm, rq);
    }
    T QI = fmaT(g.dp, g.dp, rq);
    T sF = rsq(QF), s = rsq(QI);
    T W2 = tz2 * h;
    if constexpr (MASK) W2 = (QF < thr) ? T(0) : W2;
    g.W2 = W2;
    T sF2 = sF * sF, s2 = s * s, p = sF * s;
    T Z1 = (p * (p + p)) * rcp(sF + s);
    g.Z3 = Z1 * (sF2 + p + s2);
    T s3 = s2 * s, s5 = s3 * s2;
    T base = fmaT(e2, g.Z3, Z1) - s3;
    T e2s5 = e2 * s5;
    g.cxy = fmaT(e2s5, T(3), base);
    g.cz = fmaT(e2s5, T(-3), base);
    g.s5x3 = T(3) * s5;
    return g;
}

template <typename T>
__device__ __forceinline__ void wall_apply(const WallGeo<T> &g, T f0, T f1, T f2, T *u) {
    T D = fmaT(g.d1, f1, g.d0 * f0);
    T fdF = fmaT(g.dm, f2, D);
    T P = fmaT(g.dp, f2, -D);
    T t1 = g.Z3 * fdF;
    T v = g.s5x3 * P;
    T Bxy = t1 - v;
    T u2b = fmaT(g.cz, f2, fmaT(g.dm, t1, -g.dp * v));
    u[0] = fmaT(g.W2, fmaT(g.d0, Bxy, g.cxy * f0), u[0]);
    u[1] = fmaT(g.W2, fmaT(g.d1, Bxy, g.cxy * f1), u[1]);
    u[2] = fmaT(g.W2, u2b, u[2]);
}

// Far-field wall pair in FP32 for the kernel sum, without the per-pair factor 2 t h:
// the source height h is folded into the packed strengths and 2 t is applied per
// target after each source tile, so every output accumulates with fused
// multiply-adds.  A near pair (QF < thr) gets s = 0, which zeroes every term
// exactly (the reciprocal is of sF + s >= sF > 0).  sF^2 + sF s + s^2 is formed as
// (sF + s)^2 - sF s from the reciprocal's denominator (all terms positive).
struct WallFar {
    float d0, d1, dm, dp, cxy, cz, Z3, s5x3;
};
template <bool MASK = true>
__device__ __forceinline__ WallFar wall_far_geo(float tx, float ty, float tz, float sx, float sy, float h, float e2,
                                                float thr) {
    WallFar g;
    g.d0 = sub_rn(tx, sx);
    g.d1 = sub_rn(ty, sy);
    g.dm = sub_rn(tz, h);
    g.dp = tz + h;
    const float rq = __fmaf_rn(g.d1, g.d1, __fmaf_rn(g.d0, g.d0, e2));
    const float QF = __fmaf_rn(g.dm, g.dm, rq);
    const float QI = fmaf(g.dp, g.dp, rq);
    const float sF = rsq(QF);
    float s = rsq(QI);
    if (MASK) s = (QF < thr) ? 0.0f : s;  // (MASK false: the caller knows no pair of the tile is near)
    const float p = sF * s, q = sF + s;
    const float Z1 = (p * (p + p)) * rcp(q);
    g.Z3 = Z1 * fmaf(q, q, -p);
    const float s2 = s * s, s3 = s2 * s, s5 = s3 * s2;
    const float base = fmaf(e2, g.Z3, Z1) - s3;
    const float e2s5 = e2 * s5;
    g.cxy = fmaf(e2s5, 3.0f, base);
    g.cz = fmaf(e2s5, -3.0f, base);
    g.s5x3 = 3.0f * s5;
    return g;
}
// u += the pair's velocity for the h-scaled strengths (f0, f1, f2), without the factor 2 t
__device__ __forceinline__ void wall_far_acc(const WallFar &g, float f0, float f1, float f2, float *u) {
    const float D = fmaf(g.d1, f1, g.d0 * f0);
    const float fdF = fmaf(g.dm, f2, D);
    const float P = fmaf(g.dp, f2, -D);
    const float t1 = g.Z3 * fdF;
    const float v = g.s5x3 * P;
    const float Bxy = t1 - v;
    u[0] = fmaf(g.d0, Bxy, fmaf(g.cxy, f0, u[0]));
    u[1] = fmaf(g.d1, Bxy, fmaf(g.cxy, f1, u[1]));
    u[2] = fmaf(g.cz, f2, fmaf(g.dm, t1, fmaf(-g.dp, v, u[2])));
}

// ---- two targets in one register pair (packed FP32x2 arithmetic) -------------------
// Blackwell's fma/add/sub/mul .f32x2 do two FP32 operations (one per 32-bit half, the same
// rounding as the scalar instruction) in one issue slot; the FP32 pipe's lane rate is
// unchanged, so an issue-bound pair loop gets the slots back for the pipe.  The wall
// kernel's far loop runs its two targets per thread through them, the source values
// arriving duplicated into both halves from shared memory; the special functions stay
// scalar, one per half.  Each half computes exactly what wall_far_geo / wall_far_acc
// compute for its target.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float lo2(f32x2 v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return lo;
}
__device__ __forceinline__ float hi2(f32x2 v) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return hi;
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 neg2(f32x2 a) { return a ^ 0x8000000080000000ull; }  // both signs
__device__ __forceinline__ f32x2 rsq2(f32x2 a) { return pk2(rsq(lo2(a)), rsq(hi2(a))); }
__device__ __forceinline__ f32x2 rcp2(f32x2 a) { return pk2(rcp(lo2(a)), rcp(hi2(a))); }

// u (x, y, z components, one target per half) += the far wall pair of the targets (tx, ty,
// tz) with one source (sx, sy, h, e2 and the h-scaled strengths f0, f1, f2 in both halves);
// unmasked (the caller knows no pair is near), without the factor 2 t.
__device__ __forceinline__ void wall_far_pair2(f32x2 tx, f32x2 ty, f32x2 tz, f32x2 sx, f32x2 sy, f32x2 h, f32x2 e2,
                                               f32x2 f0, f32x2 f1, f32x2 f2, f32x2 (&u)[3]) {
    const f32x2 d0 = sub2(tx, sx), d1 = sub2(ty, sy), dm = sub2(tz, h), dp = add2(tz, h);
    const f32x2 rq = fma2(d1, d1, fma2(d0, d0, e2));
    const f32x2 QF = fma2(dm, dm, rq);
    const f32x2 QI = fma2(dp, dp, rq);
    const f32x2 sF = rsq2(QF), s = rsq2(QI);
    const f32x2 p = mul2(sF, s), q = add2(sF, s);
    const f32x2 Z1 = mul2(mul2(p, add2(p, p)), rcp2(q));
    const f32x2 Z3 = mul2(Z1, fma2(q, q, neg2(p)));
    const f32x2 s2 = mul2(s, s), s3 = mul2(s2, s), s5 = mul2(s3, s2);
    const f32x2 base = sub2(fma2(e2, Z3, Z1), s3);
    const f32x2 e2s5 = mul2(e2, s5);
    const f32x2 three = 0x4040000040400000ull;  // 3.0f in both halves
    const f32x2 cxy = fma2(e2s5, three, base), cz = fma2(e2s5, neg2(three), base);
    const f32x2 s5x3 = mul2(three, s5);
    const f32x2 D = fma2(d1, f1, mul2(d0, f0));
    const f32x2 fdF = fma2(dm, f2, D);
    const f32x2 P = fma2(dp, f2, neg2(D));
    const f32x2 t1 = mul2(Z3, fdF);
    const f32x2 v = mul2(s5x3, P);
    const f32x2 Bxy = sub2(t1, v);
    u[0] = fma2(d0, Bxy, fma2(cxy, f0, u[0]));
    u[1] = fma2(d1, Bxy, fma2(cxy, f1, u[1]));
    u[2] = fma2(cz, f2, fma2(dm, t1, fma2(neg2(dp), v, u[2])));
}

}  // namespace flg
