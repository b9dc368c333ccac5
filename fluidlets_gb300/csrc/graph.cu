// graph.cu -- captured CUDA graphs of the bucket factorization (solve server).
//
// flg_bucket_graph_create captures, on the caller's stream and in thread-local
// capture mode (other host threads keep launching and allocating freely),
//   flg_assemble_bucket -> flg_convert_f64_f32 (x2: the factors' copy and the
//   inner-matvec copy A32) -> flg_lu_factor_lowp_async
// over fixed buffers, and instantiates it.  Replaying it with
// flg_graph_launch refactors whatever points are in the buffers; the real
// point count is read from device memory by the assembly kernel, so one graph
// serves every problem size of its bucket.
#include "flg_common.cuh"

extern "C" int flg_bucket_graph_create(int kind, double alpha_re, double alpha_im, const double *points,
                                       const double *eps, const int64_t *n_real, int64_t n_cap, double mu_re,
                                       double *K, float *A32, float *K32, int64_t ld32, int mode, float *dinv,
                                       int *flags, void *work, size_t work_bytes, void *stream, void **graph_exec) {
    FLG_REQUIRE(graph_exec, "null graph handle");
    FLG_REQUIRE(stream, "graph capture needs a non-default stream");
    *graph_exec = nullptr;
    cudaStream_t st = flg::as_stream(stream);
    const int64_t n = 3 * n_cap;
    // one eager pass: sets kernel attributes and any lazily initialized state outside the capture
    FLG_TRY(flg_assemble_bucket(kind, alpha_re, alpha_im, points, eps, n_real, n_cap, mu_re, K, FLG_F64, n, stream));
    FLG_TRY(flg_convert_f64_f32(n, n, K, n, K32, ld32, stream));
    if (A32) FLG_TRY(flg_convert_f64_f32(n, n, K, n, A32, ld32, stream));
    FLG_TRY(flg_lu_factor_lowp_async(n, K32, ld32, mode, dinv, flags, work, work_bytes, stream));
    FLG_CUDA(cudaStreamSynchronize(st));
    FLG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int s = flg_assemble_bucket(kind, alpha_re, alpha_im, points, eps, n_real, n_cap, mu_re, K, FLG_F64, n, stream);
    if (s == FLG_OK) s = flg_convert_f64_f32(n, n, K, n, K32, ld32, stream);
    if (s == FLG_OK && A32) s = flg_convert_f64_f32(n, n, K, n, A32, ld32, stream);
    if (s == FLG_OK) s = flg_lu_factor_lowp_async(n, K32, ld32, mode, dinv, flags, work, work_bytes, stream);
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

extern "C" int flg_graph_launch(void *graph_exec, void *stream) {
    FLG_REQUIRE(graph_exec, "null graph");
    FLG_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, flg::as_stream(stream)));
    return FLG_OK;
}

extern "C" int flg_graph_destroy(void *graph_exec) {
    if (graph_exec) FLG_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
    return FLG_OK;
}
