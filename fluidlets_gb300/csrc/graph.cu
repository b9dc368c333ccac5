// graph.cu -- captured CUDA graphs of the mixed-precision factorizations.
//
// flg_bucket_graph_create captures, on the caller's stream and in thread-local
// capture mode (other host threads keep launching and allocating freely),
//   flg_assemble_bucket -> flg_convert_f64_f32x2 (the factors' copy and the
//   inner-matvec copy A32, in one pass) -> flg_lu_factor_lowp_async
// over fixed buffers, and instantiates it (solve server).  Replaying it with
// flg_graph_launch refactors whatever points are in the buffers; the real
// point count is read from device memory by the assembly kernel, so one graph
// serves every problem size of its bucket.
//
// flg_bucket_batch_graph_create captures the same for a batch of systems of one
// bucket: one batched assembly launch, one FP32 conversion pass over all of them,
// and the batched tensor-core LU (every step's kernels cover all systems).
//
// flg_lowp_factor_graph_create captures the FP32 copies and the tensor-core LU of
// an already assembled K (resistance(), which assembles eagerly).
//
// flg_swimmer_graph_create does the same for the free-swimmer system of one
// shape size (force and quadrature point counts), for the stages of swim():
//   flg_nearest_neighbors -> flg_assemble_nearest_async ->
//   flg_swimmer_constraints_dev -> FP32 copies -> flg_lu_factor_lowp_async.
// flg_swimmer_batch_graph_create captures the same for a group of swimmer systems of
// one shape size: each system's nearest map, assembly and constraint rows, then one
// FP32 conversion pass over all of them and the batched tensor-core LU.
#include <algorithm>

#include "flg_common.cuh"

// One eager pass of `seq` (sets kernel attributes and any lazily initialized
// state outside the capture), then capture it on `stream` in thread-local mode
// and instantiate.
template <class F>
static int capture_graph(void *stream, F &&seq, void **graph_exec) {
    FLG_REQUIRE(graph_exec, "null graph handle");
    FLG_REQUIRE(stream, "graph capture needs a non-default stream");
    *graph_exec = nullptr;
    cudaStream_t st = flg::as_stream(stream);
    FLG_TRY(seq());
    FLG_CUDA(cudaStreamSynchronize(st));
    FLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int s;
    {
        flg::ProfSuppress quiet;  // no timing events inside a graph
        s = seq();
    }
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (s != FLG_OK || e != cudaSuccess || g == nullptr) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (s == FLG_OK) flg::set_error("graph capture failed: %s", cudaGetErrorString(e));
        return s != FLG_OK ? s : FLG_ERR_CUDA;
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        flg::set_error("graph instantiation failed: %s", cudaGetErrorString(e));
        return FLG_ERR_CUDA;
    }
    *graph_exec = (void *)ge;
    return FLG_OK;
}

extern "C" int flg_bucket_graph_create(int kind, double alpha_re, double alpha_im, const double *points,
                                       const double *eps, int uniform_eps, const int64_t *n_real, int64_t n_cap,
                                       double mu_re,
                                       double *K, float *A32, float *K32, int64_t ld32, int mode, float *dinv,
                                       int *flags, void *work, size_t work_bytes, void *stream, void **graph_exec) {
    FLG_RANGE("flg_bucket_graph_create");
    const int64_t n = 3 * n_cap;
    auto seq = [&]() -> int {
        if (uniform_eps)
            FLG_TRY(flg_assemble_bucket_uniform(kind, alpha_re, alpha_im, points, eps, n_real, n_cap, mu_re, K,
                                                FLG_F64, n, stream));
        else
            FLG_TRY(flg_assemble_bucket(kind, alpha_re, alpha_im, points, eps, n_real, n_cap, mu_re, K, FLG_F64, n,
                                        stream));
        FLG_TRY(flg_convert_f64_f32x2(n, n, K, n, K32, A32, ld32, stream));
        return flg_lu_factor_lowp_async(n, K32, ld32, mode, dinv, flags, work, work_bytes, stream);
    };
    return capture_graph(stream, seq, graph_exec);
}

extern "C" int flg_bucket_batch_graph_create(int kind, double alpha_re, double alpha_im, const double *points,
                                             const double *eps, int uniform_eps, const int64_t *n_real, int64_t n_cap,
                                             int nbat, double mu_re, double *K, float *A32, float *K32, int64_t ld32,
                                             int mode, float *dinv, int *flags, void *work, size_t work_bytes,
                                             void *stream, void **graph_exec) {
    FLG_RANGE("flg_bucket_batch_graph_create");
    FLG_REQUIRE(n_cap >= 1 && nbat >= 1 && ld32 >= 3 * n_cap && K && A32 && K32 && dinv && flags,
                "bad batched bucket graph arguments");
    const int64_t n = 3 * n_cap;
    auto seq = [&]() -> int {
        FLG_TRY(flg_assemble_bucket_batched(kind, alpha_re, alpha_im, points, eps, uniform_eps, n_real, n_cap, nbat,
                                            mu_re, K, FLG_F64, n, n * n, stream));
        // system z of K (n x n) and of the FP32 copies (n x ld32) are consecutive: one tall matrix
        FLG_TRY(flg_convert_f64_f32x2(nbat * n, n, K, n, K32, A32, ld32, stream));
        return flg_lu_factor_lowp_batched_async(n, nbat, K32, ld32, n * ld32, mode, dinv, flags, work, work_bytes,
                                                stream);
    };
    return capture_graph(stream, seq, graph_exec);
}

extern "C" int flg_lowp_factor_graph_create(int64_t n, const double *K, int64_t ld, float *K32, float *A32,
                                            int64_t ld32, int mode, float *dinv, int *flags, void *work,
                                            size_t work_bytes, void *stream, void **graph_exec) {
    FLG_RANGE("flg_lowp_factor_graph_create");
    FLG_REQUIRE(n >= 1 && ld >= n && ld32 >= n && K && K32 && dinv && flags, "bad factor graph arguments");
    auto seq = [&]() -> int {
        FLG_TRY(flg_convert_f64_f32x2(n, n, K, ld, K32, A32, ld32, stream));
        return flg_lu_factor_lowp_async(n, K32, ld32, mode, dinv, flags, work, work_bytes, stream);
    };
    return capture_graph(stream, seq, graph_exec);
}

extern "C" size_t flg_swimmer_graph_workspace(int64_t N, int64_t Q, int mode) {
    return std::max(flg_assemble_nearest_workspace(Q, N), flg_lu_factor_lowp_workspace(3 * N + 6, mode));
}

extern "C" int flg_swimmer_graph_create(int kind, double alpha_re, double alpha_im, const double *x, int64_t N,
                                        const double *x0, const double *X, const double *eps, int64_t Q,
                                        int64_t *nearest, int recompute_nearest, double mu_re, double *A, float *A32,
                                        float *K32, int64_t ld32, int mode, float *dinv, int *flags, void *work,
                                        size_t work_bytes, void *stream, void **graph_exec) {
    FLG_RANGE("flg_swimmer_graph_create");
    FLG_REQUIRE(N > 0 && Q >= 0 && flags && A && K32 && dinv, "bad swimmer graph arguments");
    const int64_t n = 3 * N + 6;
    FLG_REQUIRE(work_bytes >= flg_swimmer_graph_workspace(N, Q, mode), "workspace too small for the swimmer graph");
    auto seq = [&]() -> int {
        if (recompute_nearest) FLG_TRY(flg_nearest_neighbors(X, Q, x, N, nearest, stream));
        FLG_TRY(flg_assemble_nearest_async(kind, alpha_re, alpha_im, x, N, X, nearest, eps, Q, N, mu_re, 0.0, A,
                                           FLG_F64, n, flags + 2, work, work_bytes, stream));
        FLG_TRY(flg_swimmer_constraints_dev(x, N, x0, X, nearest, Q, A, FLG_F64, n, stream));
        FLG_TRY(flg_convert_f64_f32x2(n, n, A, n, K32, A32, ld32, stream));
        // the workspace is reused by the LU: the assembly is done with it by then (stream order)
        return flg_lu_factor_lowp_async(n, K32, ld32, mode, dinv, flags, work, work_bytes, stream);
    };
    return capture_graph(stream, seq, graph_exec);
}

extern "C" size_t flg_swimmer_batch_graph_workspace(int64_t N, int64_t Q, int nbat, int mode) {
    return std::max(flg_assemble_nearest_workspace(Q, N), flg_lu_factor_lowp_batched_workspace(3 * N + 6, nbat, mode));
}

extern "C" int flg_swimmer_batch_graph_create(int kind, double alpha_re, double alpha_im, const double *x, int64_t N,
                                              const double *x0, const double *X, const double *eps, int64_t Q,
                                              int64_t *nearest, int recompute_nearest, int nbat, double mu_re,
                                              double *A, float *A32, float *K32, int64_t ld32, int mode, float *dinv,
                                              int *flags, void *work, size_t work_bytes, void *stream,
                                              void **graph_exec) {
    FLG_RANGE("flg_swimmer_batch_graph_create");
    FLG_REQUIRE(N > 0 && Q >= 0 && nbat >= 1 && flags && A && K32 && dinv, "bad swimmer graph arguments");
    const int64_t n = 3 * N + 6;
    FLG_REQUIRE(ld32 >= n, "bad ld32");
    FLG_REQUIRE(work_bytes >= flg_swimmer_batch_graph_workspace(N, Q, nbat, mode),
                "workspace too small for the batched swimmer graph");
    auto seq = [&]() -> int {
        for (int z = 0; z < nbat; z++) {  // the small per-system stages, in turn on the one workspace
            const double *xz = x + 3 * N * z, *Xz = X + 3 * Q * z;
            int64_t *nz = nearest + Q * z;
            double *Az = A + n * n * z;
            if (recompute_nearest) FLG_TRY(flg_nearest_neighbors(Xz, Q, xz, N, nz, stream));
            FLG_TRY(flg_assemble_nearest_async(kind, alpha_re, alpha_im, xz, N, Xz, nz, eps + Q * z, Q, N, mu_re, 0.0,
                                               Az, FLG_F64, n, flags + 2 * nbat + z, work, work_bytes, stream));
            FLG_TRY(flg_swimmer_constraints_dev(xz, N, x0 + 3 * z, Xz, nz, Q, Az, FLG_F64, n, stream));
        }
        // system z of A (n x n) and of the FP32 copies (n x ld32) are consecutive: one tall matrix
        FLG_TRY(flg_convert_f64_f32x2(nbat * n, n, A, n, K32, A32, ld32, stream));
        return flg_lu_factor_lowp_batched_async(n, nbat, K32, ld32, n * ld32, mode, dinv, flags, work, work_bytes,
                                                stream);
    };
    return capture_graph(stream, seq, graph_exec);
}

extern "C" int flg_graph_launch(void *graph_exec, void *stream) {
    FLG_RANGE("flg_graph_launch");
    FLG_REQUIRE(graph_exec, "null graph");
    FLG_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, flg::as_stream(stream)));
    return FLG_OK;
}

extern "C" int flg_graph_destroy(void *graph_exec) {
    if (graph_exec) FLG_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
    return FLG_OK;
}
