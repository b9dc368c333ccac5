/*
 * fluidlets_gb300.h -- C ABI of libfluidlets_gb300.so (GB300, sm_103a).
 *
 * The regularized-Stokeslet hot path of the reference package `fluidlets`
 * (pure Python + Numba + SciPy): kernel sums, dense mobility-matrix assembly,
 * dense LU and matrix-free GMRES for resistance and free-swimming solves.
 *
 * Conventions (all entry points):
 *   - every pointer is a DEVICE pointer unless stated otherwise; the caller
 *     owns all memory, the library never frees caller memory;
 *   - points are (n, 3) row-major float64 ([point, component], the
 *     reference's layout, core/assemble.py:1-5); forces/velocities likewise;
 *     complex arrays are interleaved (re, im) float64 (numpy complex128);
 *   - dense matrices are row-major with a leading dimension `ld` (elements);
 *     row 3*i + a is component a of target i, column 3*j + b is component b
 *     of source j (core/assemble.py:3-5);
 *   - scratch memory is caller-provided: each entry point that needs any has
 *     a *_workspace() query returning the byte count, and takes
 *     (void* work, size_t work_bytes); a too-small workspace is FLG_ERR_INVALID;
 *   - work is enqueued on `stream` (a cudaStream_t; NULL = legacy default
 *     stream).  Entry points are asynchronous unless their comment says they
 *     synchronize (the iterative solvers read scalars back every iteration);
 *   - the return value is a status code (FLG_OK = 0).  Device code never
 *     traps; argument errors are detected on the host before any launch.
 *
 * Kernel kinds mirror the reference's kernel classes:
 *   FLG_STOKESLET      Stokeslet3D        kernels/stokeslet3d.py:53-64
 *   FLG_WALL           WallStokeslet3D    kernels/images.py:92-104
 *   FLG_BRINKMANLET    Brinkmanlet3D(a)   kernels/brinkmanlet3d.py:107-122
 *                      (alpha_im != 0 is the complex-alpha extension, which
 *                      the reference rejects at brinkmanlet3d.py:116-117)
 */
#ifndef FLUIDLETS_GB300_H
#define FLUIDLETS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define FLG_OK 0
#define FLG_ERR_INVALID 1        /* bad argument: Python raises ValueError   */
#define FLG_ERR_CUDA 2           /* CUDA runtime error (see flg_last_error)  */
#define FLG_ERR_NOT_CONVERGED 3  /* iterative solver hit maxiter: RuntimeError */
#define FLG_ERR_SINGULAR 4       /* zero / non-finite pivot: LinAlgError     */
#define FLG_ERR_NOMEM 5          /* request exceeds the caller's budget      */
#define FLG_ERR_TIMEOUT 6        /* a bounded device wait ran out: RuntimeError */

/* ---- kernel kinds, precisions, element types ---------------------------- */
#define FLG_STOKESLET 0
#define FLG_WALL 1
#define FLG_BRINKMANLET 2

#define FLG_PREC_FP64 0   /* plain FP64 everywhere: the drop-in path         */
#define FLG_PREC_MIXED 1  /* FP32 far field + FP64 near field (r < 4 eps)    */

#define FLG_F64 0
#define FLG_C128 1
#define FLG_F32 2
#define FLG_BF16 3

#define FLG_LU_TF32 0     /* tcgen05 kind::tf32, FP32 accumulate in TMEM     */
#define FLG_LU_BF16 1     /* tcgen05 kind::f16 (bf16 operands), FP32 accum   */
#define FLG_LU_FP32 2     /* FP32 CUDA cores (no tensor cores)               */
/* Optional tile-width bits OR-ed into a tensor-core LU mode: the trailing
 * updates run on 128 x 128 or 128 x 256 output tiles.  Without either bit the
 * width is chosen per update from its shape and the SM count. */
#define FLG_LU_TILE_N128 0x100
#define FLG_LU_TILE_N256 0x200

/* ---- library ------------------------------------------------------------ */
int flg_version(void);                          /* major*10000 + minor*100 + patch */
const char *flg_last_error(void);               /* thread-local message of the last failure */

/* ---- kernel sums --------------------------------------------------------
 * Replaces fluidlets.evaluate (core/matvec.py:24-49) and its Numba loop
 * _apply (core/matvec.py:10-21):  out_i = sum_j G(x_i, y_j; eps_j) f_j / mu.
 *
 *   targets (M,3) f64; sources (N,3) f64; eps (N,) f64 (a scalar eps is
 *   broadcast by the caller, core/_common.py:15-18); strengths (N,3) f64, or
 *   complex128 when strengths_complex; out (M,3) f64 or complex128 -- complex
 *   iff strengths_complex || mu_im != 0 || alpha_im != 0 (core/_common.py:21-23).
 *   precision FLG_PREC_FP64 follows the reference's FP64 arithmetic;
 *   FLG_PREC_MIXED sums pairs with r >= 4 eps_j in FP32 (per-tile FP64
 *   accumulation) and pairs with r < 4 eps_j in FP64.
 */
size_t flg_evaluate_workspace(int kind, int64_t M, int64_t N, int strengths_complex, double alpha_im,
                              int precision);
int flg_evaluate(int kind, double alpha_re, double alpha_im,
                 const double *targets, int64_t M,
                 const double *sources, const double *eps, int64_t N,
                 const double *strengths, int strengths_complex,
                 double mu_re, double mu_im,
                 double *out, int precision,
                 void *work, size_t work_bytes, void *stream);

/* Allocation-free variant of flg_evaluate, FLG_PREC_FP64 only.  No
 * counterpart in the reference: it exists for callers that cannot allocate
 * device memory at all -- a host application that reserves the whole GPU for
 * its own memory pool at start-up, or a plug-in whose framework forbids
 * cudaMalloc once it is running -- and so cannot provide the workspace of
 * flg_evaluate either.  It calls no cudaMalloc, cudaFree or other allocating
 * routine: its scratch (the per-split partial sums) is a fixed array of
 * flg_evaluate_noalloc_max_bytes() = 16 MiB of device memory that every GPU
 * loading the library holds until the process exits.  Limit: 48 bytes of
 * scratch per target with complex strengths or a complex Brinkman alpha, 24
 * bytes otherwise (a complex mu alone keeps 24), so M <= 349,525 or 699,050
 * targets; larger M returns FLG_ERR_INVALID.  The scratch is split between
 * source splits; with many targets the call runs fewer, longer splits.
 * The array is module data: under CUDA's default lazy module loading it is
 * allocated, with this file's kernels, on the first use of any of them on a
 * device.  A caller that reserves the device memory for its own pool must
 * therefore make its first call of this function (or of flg_evaluate) on each
 * device before that reservation, or run with CUDA_MODULE_LOADING=EAGER.
 * The first call on each device also looks up the array's device address
 * (with that device current) and caches it; make that first call before any
 * stream capture.  cudaDeviceReset recreates the module and invalidates the
 * cached address: do not call this function after a reset in the same process.
 * All calls share the one array and it keeps the last call's contents; calls
 * whose work overlaps on the GPU (different streams, or different host
 * threads) race: serialize them. */
size_t flg_evaluate_noalloc_max_bytes(void);
int flg_evaluate_noalloc(int kind, double alpha_re, double alpha_im,
                         const double *targets, int64_t M,
                         const double *sources, const double *eps, int64_t N,
                         const double *strengths, int strengths_complex,
                         double mu_re, double mu_im,
                         double *out, void *stream);

/* ---- dense assembly -----------------------------------------------------
 * Replaces fluidlets.assemble (core/assemble.py:27-46) and _fill (15-24):
 * K (3M x 3N) = G(x_i, y_j; eps_j) / mu written once, directly in out_type
 * (FLG_F64 | FLG_C128 | FLG_F32 | FLG_BF16; complex kernels/mu need C128),
 * row-major with leading dimension ld >= 3N.
 */
int flg_assemble(int kind, double alpha_re, double alpha_im,
                 const double *targets, int64_t M,
                 const double *sources, const double *eps, int64_t N,
                 double mu_re, double mu_im,
                 void *out, int out_type, int64_t ld, void *stream);

/* The same matrix for targets = sources (points, N) and one blob width eps,
 * from half the pair evaluations (the matrix is symmetric): for
 * FLG_STOKESLET and FLG_BRINKMANLET bit-identical to flg_assemble with
 * eps broadcast; for FLG_WALL the lower blocks are the transposes of the
 * upper ones (Lorentz reciprocity), equal to flg_assemble's to rounding. */
int flg_assemble_self_uniform(int kind, double alpha_re, double alpha_im,
                              const double *points, int64_t N, double eps,
                              double mu_re, double mu_im,
                              void *out, int out_type, int64_t ld, void *stream);

/* Assembly into a fixed-size bucket (used by the solve server's captured CUDA
 * graphs): points/eps hold n_cap entries of which the first *n_real (a DEVICE
 * int64) are real; the matrix (3 n_cap x 3 n_cap, ld) gets the kernel block
 * for real pairs and the identity for padded rows/columns, so the padded
 * system has exactly the real solution followed by zeros.  Real kernels and
 * real mu; out_type FLG_F64 or FLG_F32.  No counterpart in the reference. */
int flg_assemble_bucket(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                        const int64_t *n_real, int64_t n_cap, double mu_re, void *out, int out_type,
                        int64_t ld, void *stream);
/* The same when every point has one blob width, eps[0] (read at replay time):
 * half the pair evaluations (the mirror of block (i, j) written at (j, i) as
 * is, or transposed for the wall kernel by reciprocity, as in
 * flg_assemble_self_uniform).  No counterpart in the reference. */
int flg_assemble_bucket_uniform(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                                const int64_t *n_real, int64_t n_cap, double mu_re, void *out, int out_type,
                                int64_t ld, void *stream);
/* nbat systems of one bucket in one launch: system z has its points at
 * points + 3 z n_cap, its blob widths at eps + z n_cap, its real count at
 * n_real[z] (device) and its matrix at out + z stride_out elements
 * (stride_out >= 3 n_cap ld); uniform_eps != 0 selects the symmetric form of
 * flg_assemble_bucket_uniform (eps[z n_cap] for system z).  Each system's matrix
 * is bit-identical to its own flg_assemble_bucket(_uniform) call.  No
 * counterpart in the reference. */
int flg_assemble_bucket_batched(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                                int uniform_eps, const int64_t *n_real, int64_t n_cap, int nbat, double mu_re,
                                void *out, int out_type, int64_t ld, int64_t stride_out, void *stream);

/* Replaces fluidlets.assemble_nearest (core/assemble.py:68-101) and
 * _fill_nearest (49-58): K[:, group j] = sum_{k: nearest[k] = j} G(x_i, X_k)/mu.
 * nearest (Q,) int64 in [0, n_force).  The grouping is a deterministic
 * segmented sum (quadrature points of a group are added in ascending k).
 * out_type FLG_F64 | FLG_C128 | FLG_F32.  K is fully overwritten. */
size_t flg_assemble_nearest_workspace(int64_t Q, int64_t n_force);
int flg_assemble_nearest(int kind, double alpha_re, double alpha_im,
                         const double *targets, int64_t M,
                         const double *quad, const int64_t *nearest, const double *eps, int64_t Q,
                         int64_t n_force, double mu_re, double mu_im,
                         void *out, int out_type, int64_t ld,
                         void *work, size_t work_bytes, void *stream);
/* The same without a host synchronization (CUDA-graph capturable): *bad_flag
 * (device int, zeroed here) becomes 1 if a nearest index lies outside
 * [0, n_force); such indices are skipped.  No counterpart in the reference. */
int flg_assemble_nearest_async(int kind, double alpha_re, double alpha_im, const double *targets, int64_t M,
                               const double *quad, const int64_t *nearest, const double *eps, int64_t Q,
                               int64_t n_force, double mu_re, double mu_im, void *out, int out_type, int64_t ld,
                               int *bad_flag, void *work, size_t work_bytes, void *stream);

/* ---- free-swimmer system (swimming.py:66-102) ----------------------------
 * Fills the (3N+6) x (3N+6) system of Gallagher & Smith (2018) Eq. 8 around an
 * already assembled nearest-neighbour block A[:3N,:3N] (flg_assemble_nearest
 * with ld = 3N+6): the -U and r x Omega columns (swimming.py:92-93) and the
 * net-force / net-torque rows (95-99).  x (N,3) lab force points, x0 (3,)
 * frame origin (host pointer), X (Q,3) lab quadrature points, nearest (Q,).
 * out_type FLG_F64 | FLG_F32. */
int flg_swimmer_constraints(const double *x, int64_t N, const double *x0_host,
                            const double *X, const int64_t *nearest, int64_t Q,
                            void *A, int out_type, int64_t ld, void *stream);
/* The same with the origin x0 read from device memory (x0_dev, 3 doubles), so
 * that a captured graph picks up a new origin on every replay. */
int flg_swimmer_constraints_dev(const double *x, int64_t N, const double *x0_dev, const double *X,
                                const int64_t *nearest, int64_t Q, void *A, int out_type, int64_t ld, void *stream);

/* ---- dense LU ------------------------------------------------------------
 * Replaces the LU branch of fluidlets.resistance (core/solve.py:64-67,
 * scipy.linalg.solve = LAPACK getrf/getrs) and np.linalg.solve in
 * swimming.py:101.  Row-major A (n x n, ld), in place.
 *
 * flg_lu_factor_f64: right-looking blocked LU with partial pivoting
 * (P A = L U, unit L).  ipiv (n,) int32 device array of 0-based row swaps
 * (row k was exchanged with ipiv[k], applied in order).  info (host
 * pointer): 0, or 1 + index of the first zero pivot (then FLG_ERR_SINGULAR).
 * Synchronizes `stream`. */
size_t flg_lu_factor_f64_workspace(int64_t n);
int flg_lu_factor_f64(int64_t n, double *A, int64_t ld, int32_t *ipiv, int *info,
                      void *work, size_t work_bytes, void *stream);
/* Solves A X = B with the factors of flg_lu_factor_f64; B is (n x nrhs)
 * row-major with leading dimension ldb, overwritten by X. */
int flg_lu_solve_f64(int64_t n, int64_t nrhs, const double *LU, int64_t ld, const int32_t *ipiv,
                     double *B, int64_t ldb, void *stream);

/* Low-precision LU without pivoting for the mixed-precision path: A is FP32
 * (n x n, ld; ld a multiple of 4 so every row starts on a 16-byte boundary),
 * factored in place (unit L, U) in blocks of FLG_LU_LOWP_BLOCK.  With mode
 * FLG_LU_TF32 or FLG_LU_BF16 the panels (TF32) and the trailing updates (the
 * mode's type; rank 128 inside 512-column outer panels, rank 512 for the rest)
 * run on the tcgen05 tensor cores; FLG_LU_FP32 uses CUDA cores throughout.
 * A tensor-core mode may carry FLG_LU_TILE_N128 or FLG_LU_TILE_N256 (the tile
 * width of the trailing updates; the workspace does not depend on it).
 * dinv (FP32, size flg_lu_lowp_dinv_elems(n)) receives the inverses of the
 * diagonal blocks of L and U, used by flg_lu_solve_lowp.  Only used as a
 * preconditioner of FP64 GMRES iterative refinement, so accuracy is recovered
 * in FP64.  info as above (a zero or non-finite pivot).  Synchronizes `stream`. */
#define FLG_LU_LOWP_BLOCK 128
int64_t flg_lu_lowp_dinv_elems(int64_t n);
size_t flg_lu_factor_lowp_workspace(int64_t n, int mode);
int flg_lu_factor_lowp(int64_t n, float *A, int64_t ld, int mode, float *dinv, int *info,
                       void *work, size_t work_bytes, void *stream);
/* The same factorization without any host synchronization (so it can be
 * captured in a CUDA graph): the pivot / timeout flags are written to the
 * device array flags[2] (flags[0] = 1 + first bad pivot row, flags[1] = 1 if
 * a bounded device wait -- tensor-core pipeline or diagonal-block warps --
 * timed out) for the caller to check after the stream. */
int flg_lu_factor_lowp_async(int64_t n, float *A, int64_t ld, int mode, float *dinv, int *flags,
                             void *work, size_t work_bytes, void *stream);
/* The same for nbat (1 .. 64) independent systems of order n in one sequence
 * of launches: system z at A + z stride_a (stride_a >= n ld, a multiple of 4),
 * its block inverses at dinv + z flg_lu_lowp_dinv_elems(n), its flags at
 * flags[2 z], flags[2 z + 1] (2 nbat ints; flags[1] also reports a timed-out
 * tensor-core wait of any system).  Every kernel of a step covers all systems:
 * the diagonal blocks as one CTA per system, the panels and trailing updates
 * as one tensor-core launch over the tiles of all systems (3-D tensor maps,
 * the system index outermost).  Tensor-core modes only (TF32 / BF16, with or
 * without a tile-width bit).  Each system's factors are bit-identical to its
 * own flg_lu_factor_lowp_async call.  No counterpart in the reference. */
size_t flg_lu_factor_lowp_batched_workspace(int64_t n, int nbat, int mode);
int flg_lu_factor_lowp_batched_async(int64_t n, int nbat, float *A, int64_t ld, int64_t stride_a, int mode,
                                     float *dinv, int *flags, void *work, size_t work_bytes, void *stream);
/* x = (L U)^{-1} b in FP32 for one FP64 right-hand side (converted on the
 * fly), result written as FP64: one cooperative launch, a dataflow over the
 * 128-row blocks with bounded waits (a timed-out wait makes x NaN). */
size_t flg_lu_solve_lowp_workspace(int64_t n);
int flg_lu_solve_lowp(int64_t n, const float *LU, int64_t ld, const float *dinv, const double *b, double *x,
                      void *work, size_t work_bytes, void *stream);

/* Tensor-core rank-128 update used by the trailing updates of
 * flg_lu_factor_lowp, exposed as a building block:
 *   C (m x nc, FP32, ldc)  -=  A (m x 128, FP32, lda) * Bt^T,  Bt (nc x 128, FP32, ldb = 128)
 * mode FLG_LU_TF32 (kind::tf32) or FLG_LU_BF16 (operands rounded to BF16,
 * kind::f16); FP32 accumulation in TMEM.  A and C rows must start on 16-byte
 * boundaries (lda, ldc multiples of 4).  Synchronizes `stream`. */
size_t flg_tc_rank_update_workspace(int64_t m, int64_t nc, int mode);
int flg_tc_rank_update(float *C, int64_t ldc, const float *A, int64_t lda, const float *Bt, int64_t ldb,
                       int64_t m, int64_t nc, int mode, void *work, size_t work_bytes, void *stream);

/* ---- GMRES ---------------------------------------------------------------
 * Restarted GMRES with the semantics of scipy.sparse.linalg.gmres as called
 * by fluidlets.resistance (core/solve.py:68-79): rtol relative to ||b||,
 * atol = 0, `restart` inner iterations, `maxiter` restart cycles, adaptive
 * inner tolerance (scipy gh-8400), iteration count = number of inner
 * iterations (callback_type "pr_norm").  Orthogonalization is classical
 * Gram-Schmidt with one re-orthogonalization (CGS2).
 *
 * Matrix-free operator: A v = evaluate(kind, X, X, v, eps, mu) (n = 3N
 * unknowns, real or complex).  precision:
 *   FLG_PREC_FP64  plain FP64 matvec throughout;
 *   FLG_PREC_MIXED iterative refinement: FP64 outer residual b - A x, inner
 *                  GMRES on FLG_PREC_MIXED matvecs to inner_rtol.
 * x (3N) in/out (initial guess; zero for the reference's behaviour).
 * iters/outer/resid are host pointers: inner iterations, outer refinement
 * steps, final ||b - A x|| / ||b|| (FP64 operator).  Synchronizes `stream`. */
size_t flg_gmres_workspace(int64_t N, int restart, int is_complex, int precision);
int flg_gmres(int kind, double alpha_re, double alpha_im,
              const double *X, const double *eps, int64_t N,
              double mu_re, double mu_im,
              const double *b, double *x, int is_complex,
              double rtol, int restart, int maxiter, int precision, double inner_rtol,
              int *iters, int *outer, double *resid,
              void *work, size_t work_bytes, void *stream);

/* Dense GMRES-IR: solves A x = b (n x n FP64 row-major, ld) to rtol with
 * FP64 residuals b - A x (FP64 GEMV), correcting with inner GMRES (tolerance
 * 1e-4) on the operator M^-1 A, M = the low-precision factors of
 * flg_lu_factor_lowp (LU32, ld32, dinv).  The inner matvecs use A32 (an FP32
 * copy of A, leading dimension lda32) when it is not NULL, else A.  Real
 * only.  iters = total inner iterations, outer = refinement steps, resid =
 * final ||b - A x|| / ||b|| with the FP64 A.  Synchronizes. */
size_t flg_gmres_ir_dense_workspace(int64_t n, int restart);
int flg_gmres_ir_dense(int64_t n, const double *A, int64_t ld, const float *A32, int64_t lda32,
                       const float *LU32, int64_t ld32, const float *dinv, const double *b, double *x,
                       double rtol, int restart, int maxiter, int *iters, int *outer, double *resid,
                       void *work, size_t work_bytes, void *stream);

/* ---- captured graphs (solve server) ---------------------------------------
 * Captures flg_assemble_bucket -> flg_convert_f64_f32 -> flg_lu_factor_lowp_async
 * over fixed buffers (K: 3 n_cap x 3 n_cap FP64; A32 (optional) and K32, FP32 copies
 * with ld32, the second factored in place; dinv, flags[2],
 * LU workspace) on `stream` (not the default stream) in thread-local capture
 * mode, after one eager pass, and returns the instantiated graph.  Replay with
 * flg_graph_launch; the real point count is read from *n_real at replay time.
 * uniform_eps != 0: every point has the blob width eps[0] (read at replay time)
 * and the assembly is flg_assemble_bucket_uniform, from half the pairs.
 * No counterpart in the reference. */
int flg_bucket_graph_create(int kind, double alpha_re, double alpha_im, const double *points, const double *eps,
                            int uniform_eps, const int64_t *n_real, int64_t n_cap, double mu_re, double *K,
                            float *A32, float *K32,
                            int64_t ld32, int mode, float *dinv, int *flags, void *work, size_t work_bytes,
                            void *stream, void **graph_exec);
/* The batched form of flg_bucket_graph_create: nbat systems of one bucket
 * (points, eps, n_real laid out as in flg_assemble_bucket_batched), K system z
 * at K + z 9 n_cap^2 (ld 3 n_cap), A32 / K32 system z at + z 3 n_cap ld32,
 * dinv and flags as in flg_lu_factor_lowp_batched_async, workspace
 * flg_lu_factor_lowp_batched_workspace(3 n_cap, nbat, mode).  One graph:
 * flg_assemble_bucket_batched -> one FP32 conversion pass over all systems ->
 * flg_lu_factor_lowp_batched_async.  No counterpart in the reference. */
int flg_bucket_batch_graph_create(int kind, double alpha_re, double alpha_im, const double *points,
                                  const double *eps, int uniform_eps, const int64_t *n_real, int64_t n_cap, int nbat,
                                  double mu_re, double *K, float *A32, float *K32, int64_t ld32, int mode,
                                  float *dinv, int *flags, void *work, size_t work_bytes, void *stream,
                                  void **graph_exec);
/* The FP32 copies (flg_convert_f64_f32x2) and the tensor-core LU
 * (flg_lu_factor_lowp_async) of an assembled FP64 K as one captured graph over
 * fixed buffers (replay with flg_graph_launch; flags as in
 * flg_lu_factor_lowp_async).  No counterpart in the reference. */
int flg_lowp_factor_graph_create(int64_t n, const double *K, int64_t ld, float *K32, float *A32, int64_t ld32,
                                 int mode, float *dinv, int *flags, void *work, size_t work_bytes, void *stream,
                                 void **graph_exec);
/* Captured graph of the free-swimmer system (swimming.py:66-102) for N force
 * points and Q quadrature points, over fixed device buffers: x (N x 3), x0 (3),
 * X (Q x 3), eps (Q), nearest (Q; recomputed from x and X on every replay when
 * recompute_nearest != 0) -> A ((3N+6)^2 FP64, ld 3N+6) -> FP32 copies A32
 * (optional) and K32 (ld32) -> tensor-core LU of K32 with dinv.  flags[0..1]
 * as flg_lu_factor_lowp_async, flags[2] = 1 on an invalid nearest index.
 * Workspace: flg_swimmer_graph_workspace(N, Q, mode).  Each stage of swim()
 * writes its points into the buffers and replays the graph. */
size_t flg_swimmer_graph_workspace(int64_t N, int64_t Q, int mode);
int flg_swimmer_graph_create(int kind, double alpha_re, double alpha_im, const double *x, int64_t N,
                             const double *x0, const double *X, const double *eps, int64_t Q, int64_t *nearest,
                             int recompute_nearest, double mu_re, double *A, float *A32, float *K32, int64_t ld32,
                             int mode, float *dinv, int *flags, void *work, size_t work_bytes, void *stream,
                             void **graph_exec);
/* The batched form for a group of nbat swimmer systems of one shape size: system z has
 * x + 3 N z, x0 + 3 z, X + 3 Q z, eps + Q z, nearest + Q z, A + z (3N+6)^2 (ld 3N+6), A32 / K32
 * + z (3N+6) ld32, dinv + z flg_lu_lowp_dinv_elems(3N+6); flags holds 3 nbat ints: the LU
 * flags of system z at flags[2 z], flags[2 z + 1] (as flg_lu_factor_lowp_batched_async) and its
 * invalid-nearest-index flag at flags[2 nbat + z] (nbat = 1: the layout of
 * flg_swimmer_graph_create).  One graph: each system's nearest map (when recompute_nearest),
 * nearest-neighbour assembly and constraint rows, then one FP32 conversion pass over all
 * systems and flg_lu_factor_lowp_batched_async (tensor-core modes).  Each system's factors are
 * bit-identical to its own flg_swimmer_graph_create replay.  No counterpart in the reference. */
size_t flg_swimmer_batch_graph_workspace(int64_t N, int64_t Q, int nbat, int mode);
int flg_swimmer_batch_graph_create(int kind, double alpha_re, double alpha_im, const double *x, int64_t N,
                                   const double *x0, const double *X, const double *eps, int64_t Q, int64_t *nearest,
                                   int recompute_nearest, int nbat, double mu_re, double *A, float *A32, float *K32,
                                   int64_t ld32, int mode, float *dinv, int *flags, void *work, size_t work_bytes,
                                   void *stream, void **graph_exec);
int flg_graph_launch(void *graph_exec, void *stream);
int flg_graph_destroy(void *graph_exec);

/* Nearest force point of each quadrature point: out[q] = argmin_j |quad_q - force_j|
 * (FP64, first index on ties); replaces the k-d tree query of
 * core/assemble.py:61-65 (nearest_neighbors).  Exhaustive, O(Q N). */
int flg_nearest_neighbors(const double *quad, int64_t Q, const double *force, int64_t N, int64_t *out, void *stream);

/* ---- geometry on the device --------------------------------------------------
 * The reference's sphere discretizations, same arithmetic in the same order:
 * flg_fibonacci_sphere writes n points (geometry/spheres.py:7-13, golden-angle
 * spiral), flg_cube_sphere 6 n^2 points (geometry/spheres.py:33-52, six-patch
 * sphere); center is a host array of 3, out (device) is (points x 3) FP64.
 * flg_mean_nn_spacing: the mean distance from each point to its nearest other
 * point (*mean on the device; workspace flg_mean_nn_spacing_workspace(n)),
 * which the workloads use to choose blob widths. */
int flg_fibonacci_sphere(int64_t n, double radius, const double *center, double *out, void *stream);
int flg_cube_sphere(int64_t n, double radius, const double *center, double *out, void *stream);
size_t flg_mean_nn_spacing_workspace(int64_t n);
int flg_mean_nn_spacing(const double *points, int64_t n, double *mean, void *work, size_t work_bytes, void *stream);

/* ---- structured grids ----------------------------------------------------
 * points (nx ny nz x 3, FP64) of the grid x_axis x y_axis x z_axis (device
 * arrays), x fastest, then y, then z: the point order of the reference's
 * examples (np.meshgrid(z, y, x, indexing="ij") raveled, e.g.
 * examples/glycocalyx_towers/run.py:48-51) and of VTK structured grids.  A
 * velocity field evaluated at these points (flg_evaluate) is in VTK order. */
int flg_grid_points(const double *x_axis, int64_t nx, const double *y_axis, int64_t ny, const double *z_axis,
                    int64_t nz, double *points, void *stream);

/* ---- dense helpers --------------------------------------------------------
 * y = A x (FP64, row-major n_rows x n_cols, ld); used for residuals. */
int flg_gemv_f64(int64_t n_rows, int64_t n_cols, const double *A, int64_t ld, const double *x, double *y,
                 void *stream);
/* y (FP64) = A (FP32, row-major n_rows x n_cols, ld) x (FP64), computed with
 * compensated FP32 arithmetic (x split into two FP32 parts, error-free products
 * and sums) to about FP64 accuracy for the given FP32 entries: the inner matvec
 * of GMRES-IR.  No counterpart in the reference. */
int flg_gemv_f32(int64_t n_rows, int64_t n_cols, const float *A, int64_t ld, const double *x, double *y,
                 void *stream);
/* dst (FP32, ldd) = (float) src (FP64, lds), n_rows x n_cols */
int flg_convert_f64_f32(int64_t n_rows, int64_t n_cols, const double *src, int64_t lds, float *dst, int64_t ldd,
                        void *stream);
/* dst1 = dst2 = (float) src in one pass over src (dst2 may be NULL): the mixed
 * solve's factored copy and inner-matvec copy.  No counterpart in the reference. */
int flg_convert_f64_f32x2(int64_t n_rows, int64_t n_cols, const double *src, int64_t lds, float *dst1, float *dst2,
                          int64_t ldd, void *stream);

/* FP64 GMRES-based iterative refinement of K x = b (the same algorithm as
 * flg_gmres_ir_dense, with one restart cycle of at most m inner columns per
 * refinement step) as one instantiated CUDA graph over fixed buffers: the
 * refinement and inner loops are conditional WHILE nodes whose conditions
 * single-thread control kernels set on the device, and every scalar (norms,
 * Hessenberg matrix, rotations) stays in device memory, so a replay
 * (flg_graph_launch) costs no host round trip.  Tolerance rtol on
 * ||b - K x|| / ||b|| with the FP64 K; at most max_outer refinement steps;
 * m <= 64.  The workspace (flg_gmres_ir_graph_workspace) belongs to the graph;
 * flg_gmres_ir_graph_result reads the last replay's outcome from it
 * (synchronizes): FLG_OK, or FLG_ERR_NOT_CONVERGED on stagnation or the step
 * limit.  The creating stream must be a non-default stream.  No counterpart in
 * the reference (its solves run on the host, core/solve.py:64-79). */
size_t flg_gmres_ir_graph_workspace(int64_t n, int m);
int flg_gmres_ir_graph_create(int64_t n, const double *K, int64_t ld, const float *A32, int64_t lda32,
                              const float *LU32, int64_t ld32, const float *dinv, const double *b, double *x,
                              double rtol, int m, int max_outer, void *work, size_t work_bytes, void *stream,
                              void **graph_exec);
int flg_gmres_ir_graph_result(const void *work, int *iters, int *outer, double *resid, void *stream);

/* ---- measurement ----------------------------------------------------------
 * Throughput microbenchmarks used as roofline denominators (FFMA FP32, DFMA
 * FP64), in TFLOP/s, timed with CUDA events on `stream`.  Synchronizes. */
int flg_measure_peaks(double *fp32_tflops, double *fp64_tflops, void *stream);

/* Kernel timing and launch counting (measurement aid; off by default).
 * While enabled, the library records a CUDA event pair on the launching
 * stream around every launch of the profiled kernels below, and counts every
 * kernel it launches.  flg_profile_enable(1) resets the records.
 * flg_profile_read synchronizes the recorded events and returns the total
 * milliseconds and launch count of one slot.  Process-wide state: enable it
 * only around a measurement. */
#define FLG_SLOT_FAR_F32 0      /* far_f32_kernel (mixed-precision far field)  */
#define FLG_SLOT_NEAR_F64 1     /* near_f64_kernel (near field + combine)       */
#define FLG_SLOT_SUM_F64 2      /* sum_f64_kernel (plain FP64 sum)              */
#define FLG_SLOT_ASSEMBLE 3     /* dense assembly kernels                       */
#define FLG_SLOT_LU_UPDATE 4    /* LU trailing updates (tensor-core GEMM)       */
#define FLG_SLOT_LU_PANEL 5     /* LU panel kernels (FP64 panel; low-precision L21 / U12) */
#define FLG_SLOT_GEMV 6         /* FP64 GEMV (residuals)                        */
#define FLG_SLOT_LU_SOLVE 7     /* low-precision triangular solves (preconditioner) */
#define FLG_SLOT_LU_DIAG 8      /* low-precision LU diagonal-block factor + inverses */
#define FLG_NUM_SLOTS 9
int flg_profile_enable(int enable);
int flg_profile_read(int slot, double *total_ms, int64_t *launches);
int64_t flg_launch_count(void);

/* ---- failure detection ----------------------------------------------------
 * Every spin-wait in the library's kernels is bounded (2 s in production) and
 * reports a wait that ran out as FLG_ERR_TIMEOUT instead of hanging the GPU.
 * No counterpart in the reference (its solvers run on the host; their only
 * failure report is RuntimeError on GMRES non-convergence, core/solve.py:77-78).
 * flg_wait_selftest drives one kind of wait to expiry on a condition nothing
 * satisfies, with a limit of `limit_ms`: which = 0 the grid barrier of the FP64
 * LU panel (one arrival never comes), 1 the low-precision solve's poll of a
 * published value (nothing publishes it), 2 the tensor-core update's mbarrier
 * wait (no arrival completes the phase).  It returns FLG_ERR_TIMEOUT, as the
 * production entry points do for such a wait, after about limit_ms, with the
 * context still usable.  Synchronizes. */
size_t flg_wait_selftest_workspace(void);
int flg_wait_selftest(int which, double limit_ms, void *work, size_t work_bytes, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDLETS_GB300_H */
