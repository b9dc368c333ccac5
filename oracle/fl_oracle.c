/*
 * fl_oracle.c -- CPU restatement of the reference's FP64 kernel arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path of
 * fluidlets_gb300 is checked against.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arms may load it.  The product
 * library never links or calls it.
 *
 * Every function restates the reference (fluidlets, pure Python + Numba) in
 * plain C with the same operation order, so that results agree with the
 * reference to the last few ulps:
 *
 *   stokeslet_block   kernels/stokeslet3d.py:22-50   (H1, H2, block)
 *   image_block       kernels/images.py:26-78        (Ainley et al. 2008 image system)
 *   wall_block        kernels/images.py:81-89        (image + free Stokeslet)
 *   brink_f1/f2       kernels/brinkmanlet3d.py:43-71 (24-term series below z = 0.5)
 *   brink_block       kernels/brinkmanlet3d.py:74-104
 *   orc_apply         core/matvec.py:10-21           (_apply: prange over targets)
 *   orc_fill          core/assemble.py:15-24         (_fill)
 *   orc_fill_nearest  core/assemble.py:49-58         (_fill_nearest)
 *
 * Complex Brinkman alpha is not supported by the reference (it raises,
 * kernels/brinkmanlet3d.py:116-117).  The complex branch here is the same
 * formula with z = alpha R complex, series when |z| < 0.5; its parity is
 * pinned against mpmath (tests/test_oracle.py), not against the reference.
 *
 * Build: cc -O2 -fopenmp -fPIC -shared fl_oracle.c -o _build/liboracle.so -lm
 * (no -ffast-math: the oracle must keep IEEE semantics).
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { ORC_STOKESLET = 0, ORC_WALL = 1, ORC_BRINKMAN = 2 };

#define ORC_PI 3.141592653589793

/* ---- regularized Stokeslet: kernels/stokeslet3d.py:22-50 ---------------- */
static inline double st_H1(double r2, double eps2) {
    return (r2 + 2.0 * eps2) / (8.0 * ORC_PI * pow(r2 + eps2, 1.5));
}
static inline double st_H2(double r2, double eps2) {
    return 1.0 / (8.0 * ORC_PI * pow(r2 + eps2, 1.5));
}
static void stokeslet_block(const double *x, const double *x0, double eps, double *out) {
    double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] - x0[2];
    double r2 = d0 * d0 + d1 * d1 + d2 * d2;
    double eps2 = eps * eps;
    double h1 = st_H1(r2, eps2), h2 = st_H2(r2, eps2);
    out[0] = h1 + h2 * d0 * d0;
    out[1] = h2 * d0 * d1;
    out[2] = h2 * d0 * d2;
    out[3] = out[1];
    out[4] = h1 + h2 * d1 * d1;
    out[5] = h2 * d1 * d2;
    out[6] = out[2];
    out[7] = out[5];
    out[8] = h1 + h2 * d2 * d2;
}

/* ---- wall image system: kernels/images.py:26-78 -------------------------- */
static void image_block(const double *x, const double *x0, double eps, double *out) {
    double h0 = x0[2];
    double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] + h0;
    double eps2 = eps * eps;
    double Q = d0 * d0 + d1 * d1 + d2 * d2 + eps2;
    double q1 = pow(Q, 0.5), q3 = pow(Q, 1.5), q5 = pow(Q, 2.5);
    double H1 = 0.5 / q1 + 0.5 * eps2 / q3;
    double H2 = 0.5 / q3;
    double Hdp1 = -h0 * h0 * (1.0 / q3 - 3.0 * eps2 / q5);
    double Hdp2 = -h0 * h0 * (-3.0 / q5);
    double Hdb1 = 2.0 * h0 * (-1.5 * eps2 / q5 - 0.5 / q3);
    double Hdb2 = 2.0 * h0 * (0.5 / q3);
    double Hdb3 = 2.0 * h0 * (-1.5 / q5);
    double Hr1 = h0 * 3.0 * eps2 / q5;
    double d[3] = {d0, d1, d2};
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double delta = (i == j) ? 1.0 : 0.0;
            double a = -(delta * H1 + d[i] * d[j] * H2);
            double sgn = (j == 2) ? 1.0 : -1.0;
            a += sgn * (delta * Hdp1 + d[i] * d[j] * Hdp2);
            out[3 * i + j] = a;
        }
    out[0] -= d2 * (Hdb2 + d0 * d0 * Hdb3);
    out[1] -= d0 * d1 * d2 * Hdb3;
    out[2] += d0 * (Hdb2 + d2 * d2 * Hdb3);
    out[3] -= d1 * d0 * d2 * Hdb3;
    out[4] -= d2 * (Hdb2 + d1 * d1 * Hdb3);
    out[5] += d1 * (Hdb2 + d2 * d2 * Hdb3);
    out[6] -= d0 * (Hdb1 + d2 * d2 * Hdb3);
    out[7] -= d1 * (Hdb1 + d2 * d2 * Hdb3);
    out[8] += d2 * (Hdb1 + 2.0 * Hdb2 + d2 * d2 * Hdb3);
    out[0] += d2 * Hr1;
    out[4] += d2 * Hr1;
    out[6] -= d0 * Hr1;
    out[7] -= d1 * Hr1;
    for (int k = 0; k < 9; k++) out[k] /= 4.0 * ORC_PI;
}

/* kernels/images.py:81-89: image part, then the free Stokeslet added on top */
static void wall_block(const double *x, const double *x0, double eps, double *out) {
    double tmp[9];
    image_block(x, x0, eps, out);
    stokeslet_block(x, x0, eps, tmp);
    for (int k = 0; k < 9; k++) out[k] += tmp[k];
}

/* ---- Brinkmanlet: kernels/brinkmanlet3d.py:43-104 ----------------------- */
#define BR_NTERMS 24
#define BR_ZSERIES 0.5
static double BR_C1[BR_NTERMS], BR_C2[BR_NTERMS];
static int br_init_done = 0;

static void br_init(void) {
    if (br_init_done) return;
    /* C1[n] = (-1)^n (1/(n+2)! - 1/(n+1)! + 1/n!)
       C2[n] = (-1)^(n+1) (3/(n+2)! - 3/(n+1)! + 1/n!)      (brinkmanlet3d.py:46-49) */
    long double fact[BR_NTERMS + 3];
    fact[0] = 1.0L;
    for (int k = 1; k < BR_NTERMS + 3; k++) fact[k] = fact[k - 1] * (long double)k;
    for (int n = 0; n < BR_NTERMS; n++) {
        double a = (double)(1.0L / fact[n + 2]), b = (double)(1.0L / fact[n + 1]), c = (double)(1.0L / fact[n]);
        double s = (n % 2 == 0) ? 1.0 : -1.0;
        BR_C1[n] = s * (a - b + c);
        BR_C2[n] = -s * (3.0 * a - 3.0 * b + c);
    }
    br_init_done = 1;
}

static inline double brink_f1(double z) {
    if (z < BR_ZSERIES) {
        double s = 0.0;
        for (int n = BR_NTERMS - 1; n >= 0; n--) s = s * z + BR_C1[n];
        return s;
    }
    return exp(-z) * (1.0 + 1.0 / z + 1.0 / (z * z)) - 1.0 / (z * z);
}
static inline double brink_f2(double z) {
    if (z < BR_ZSERIES) {
        double s = 0.0;
        for (int n = BR_NTERMS - 1; n >= 0; n--) s = s * z + BR_C2[n];
        return s;
    }
    return 3.0 / (z * z) - exp(-z) * (1.0 + 3.0 / z + 3.0 / (z * z));
}
static void brink_block(const double *x, const double *x0, double eps, double alpha, double *out) {
    double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] - x0[2];
    double r2 = d0 * d0 + d1 * d1 + d2 * d2, eps2 = eps * eps;
    double R = sqrt(r2 + eps2);
    double z = alpha * R;
    double h1 = brink_f1(z) / (4.0 * ORC_PI * R);
    double h2 = brink_f2(z) / (4.0 * ORC_PI * R * R * R);
    double H1 = h1 + eps2 * h2, H2 = h2;
    out[0] = H1 + H2 * d0 * d0;
    out[1] = H2 * d0 * d1;
    out[2] = H2 * d0 * d2;
    out[3] = out[1];
    out[4] = H1 + H2 * d1 * d1;
    out[5] = H2 * d1 * d2;
    out[6] = out[2];
    out[7] = out[5];
    out[8] = H1 + H2 * d2 * d2;
}

/* complex alpha: same formula, z = alpha R complex; series when |z| < 0.5 */
static inline double complex brink_f1c(double complex z) {
    if (cabs(z) < BR_ZSERIES) {
        double complex s = 0.0;
        for (int n = BR_NTERMS - 1; n >= 0; n--) s = s * z + BR_C1[n];
        return s;
    }
    return cexp(-z) * (1.0 + 1.0 / z + 1.0 / (z * z)) - 1.0 / (z * z);
}
static inline double complex brink_f2c(double complex z) {
    if (cabs(z) < BR_ZSERIES) {
        double complex s = 0.0;
        for (int n = BR_NTERMS - 1; n >= 0; n--) s = s * z + BR_C2[n];
        return s;
    }
    return 3.0 / (z * z) - cexp(-z) * (1.0 + 3.0 / z + 3.0 / (z * z));
}
static void brink_block_c(const double *x, const double *x0, double eps, double complex alpha,
                          double complex *out) {
    double d0 = x[0] - x0[0], d1 = x[1] - x0[1], d2 = x[2] - x0[2];
    double r2 = d0 * d0 + d1 * d1 + d2 * d2, eps2 = eps * eps;
    double R = sqrt(r2 + eps2);
    double complex z = alpha * R;
    double complex h1 = brink_f1c(z) / (4.0 * ORC_PI * R);
    double complex h2 = brink_f2c(z) / (4.0 * ORC_PI * R * R * R);
    double complex H1 = h1 + eps2 * h2, H2 = h2;
    out[0] = H1 + H2 * d0 * d0;
    out[1] = H2 * d0 * d1;
    out[2] = H2 * d0 * d2;
    out[3] = out[1];
    out[4] = H1 + H2 * d1 * d1;
    out[5] = H2 * d1 * d2;
    out[6] = out[2];
    out[7] = out[5];
    out[8] = H1 + H2 * d2 * d2;
}

/* params: [alpha_re, alpha_im] for ORC_BRINKMAN, unused otherwise */
static inline int is_complex_kernel(int kind, const double *params) {
    return kind == ORC_BRINKMAN && params && params[1] != 0.0;
}

/* One 3x3 block, complex in general (imaginary part 0 for real kernels). */
static void block_c(int kind, const double *params, const double *x, const double *x0, double eps,
                    double complex *G) {
    if (is_complex_kernel(kind, params)) {
        brink_block_c(x, x0, eps, params[0] + I * params[1], G);
        return;
    }
    double g[9];
    if (kind == ORC_STOKESLET) stokeslet_block(x, x0, eps, g);
    else if (kind == ORC_WALL) wall_block(x, x0, eps, g);
    else brink_block(x, x0, eps, params ? params[0] : 0.0, g);
    for (int k = 0; k < 9; k++) G[k] = g[k];
}

static void block_r(int kind, const double *params, const double *x, const double *x0, double eps, double *g) {
    if (kind == ORC_STOKESLET) stokeslet_block(x, x0, eps, g);
    else if (kind == ORC_WALL) wall_block(x, x0, eps, g);
    else brink_block(x, x0, eps, params ? params[0] : 0.0, g);
}

static void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* Exported: the single 3x3 block (row-major), complex interleaved (re, im). */
void orc_block(int kind, const double *params, const double *x, const double *x0, double eps, double *G_ri) {
    br_init();
    double complex G[9];
    block_c(kind, params, x, x0, eps, G);
    for (int k = 0; k < 9; k++) {
        G_ri[2 * k] = creal(G[k]);
        G_ri[2 * k + 1] = cimag(G[k]);
    }
}

void orc_brink_f(double z_re, double z_im, double *f1_ri, double *f2_ri) {
    br_init();
    if (z_im == 0.0) {
        f1_ri[0] = brink_f1(z_re); f1_ri[1] = 0.0;
        f2_ri[0] = brink_f2(z_re); f2_ri[1] = 0.0;
        return;
    }
    double complex z = z_re + I * z_im;
    double complex a = brink_f1c(z), b = brink_f2c(z);
    f1_ri[0] = creal(a); f1_ri[1] = cimag(a);
    f2_ri[0] = creal(b); f2_ri[1] = cimag(b);
}

/*
 * core/matvec.py:10-21 (_apply).  Targets (M,3), sources (N,3), eps (N,),
 * strengths (N,3) real or complex-interleaved, out (M,3) zero-initialised by
 * the caller in the same dtype (real unless f or the kernel is complex).
 * Accumulation order per target row follows the reference exactly:
 * out[i,a] += sum_b G[a,b] f[j,b], j ascending.
 */
void orc_apply(int kind, const double *params, int64_t M, const double *tg, int64_t N, const double *src,
               const double *eps, const double *f, int f_complex, double *out, int nthreads) {
    br_init();
    set_threads(nthreads);
    int cplx = f_complex || is_complex_kernel(kind, params);
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < M; i++) {
        if (!cplx) {
            double G[9];
            for (int64_t j = 0; j < N; j++) {
                block_r(kind, params, tg + 3 * i, src + 3 * j, eps[j], G);
                for (int a = 0; a < 3; a++) {
                    double acc = out[3 * i + a] * 0.0;
                    for (int b = 0; b < 3; b++) acc += G[3 * a + b] * f[3 * j + b];
                    out[3 * i + a] += acc;
                }
            }
        } else {
            double complex G[9];
            double complex *o = (double complex *)out;
            for (int64_t j = 0; j < N; j++) {
                block_c(kind, params, tg + 3 * i, src + 3 * j, eps[j], G);
                for (int a = 0; a < 3; a++) {
                    double complex acc = o[3 * i + a] * 0.0;
                    for (int b = 0; b < 3; b++) {
                        double complex fb = f_complex ? (f[6 * j + 2 * b] + I * f[6 * j + 2 * b + 1])
                                                      : (double complex)f[3 * j + b];
                        acc += G[3 * a + b] * fb;
                    }
                    o[3 * i + a] += acc;
                }
            }
        }
    }
}

/* core/assemble.py:15-24 (_fill).  K is (3M) x (3N), real or complex-interleaved. */
void orc_fill(int kind, const double *params, int64_t M, const double *tg, int64_t N, const double *src,
              const double *eps, double *K, int nthreads) {
    br_init();
    set_threads(nthreads);
    int cplx = is_complex_kernel(kind, params);
    int64_t ld = 3 * N;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t j = 0; j < N; j++) {
            if (!cplx) {
                double G[9];
                block_r(kind, params, tg + 3 * i, src + 3 * j, eps[j], G);
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) K[(3 * i + a) * ld + 3 * j + b] = G[3 * a + b];
            } else {
                double complex G[9];
                block_c(kind, params, tg + 3 * i, src + 3 * j, eps[j], G);
                double complex *Kc = (double complex *)K;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) Kc[(3 * i + a) * ld + 3 * j + b] = G[3 * a + b];
            }
        }
    }
}

/* core/assemble.py:49-58 (_fill_nearest).  K zero-initialised by the caller,
   (3M) x (3*n_force); quadrature point k adds its block to column group nearest[k]. */
void orc_fill_nearest(int kind, const double *params, int64_t M, const double *tg, int64_t Q, const double *quad,
                      const int64_t *nearest, const double *eps, int64_t n_force, double *K, int nthreads) {
    br_init();
    set_threads(nthreads);
    int cplx = is_complex_kernel(kind, params);
    int64_t ld = 3 * n_force;
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < M; i++) {
        for (int64_t k = 0; k < Q; k++) {
            int64_t j = nearest[k];
            if (!cplx) {
                double G[9];
                block_r(kind, params, tg + 3 * i, quad + 3 * k, eps[k], G);
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) K[(3 * i + a) * ld + 3 * j + b] += G[3 * a + b];
            } else {
                double complex G[9];
                block_c(kind, params, tg + 3 * i, quad + 3 * k, eps[k], G);
                double complex *Kc = (double complex *)K;
                for (int a = 0; a < 3; a++)
                    for (int b = 0; b < 3; b++) Kc[(3 * i + a) * ld + 3 * j + b] += G[3 * a + b];
            }
        }
    }
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
