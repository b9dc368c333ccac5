// peaks.cu -- FP32 / FP64 throughput microbenchmarks (roofline denominators).
//
// MEASURED_PEAKS-style numbers for the pipes the kernel sums use: independent
// FFMA (FP32) and DFMA (FP64) chains, 8 per thread, 8 CTAs of 256 threads per
// SM.  FLOPs = 2 per fused multiply-add.
#include "flg_common.cuh"

namespace flg {

template <typename T, int CH>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *sink, int iters, T a, T b) {
    T x[CH];
#pragma unroll
    for (int c = 0; c < CH; c++) x[c] = T(threadIdx.x) * T(1e-3) + T(c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < CH; c++) x[c] = fma(x[c], a, b);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < CH; c++) s += x[c];
    if (s == T(1234.5)) sink[0] = s;  // never true; keeps the chains live
}

template <typename T>
static int time_fma(int iters, double *tflops, cudaStream_t st) {
    const int sms = sm_count(), blocks = sms * 8, threads = 256;
    T *sink;
    FLG_CUDA(cudaMallocAsync(&sink, 64, st));
    cudaEvent_t e0, e1;
    FLG_CUDA(cudaEventCreate(&e0));
    FLG_CUDA(cudaEventCreate(&e1));
    fma_chain_kernel<T, 8><<<blocks, threads, 0, st>>>(sink, iters / 20 + 1, T(1.0001), T(1e-4));  // warm-up
    FLG_LAUNCH_CHECK();
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        FLG_CUDA(cudaEventRecord(e0, st));
        fma_chain_kernel<T, 8><<<blocks, threads, 0, st>>>(sink, iters, T(1.0001), T(1e-4));
        FLG_LAUNCH_CHECK();
        FLG_CUDA(cudaEventRecord(e1, st));
        FLG_CUDA(cudaEventSynchronize(e1));
        float ms;
        FLG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = ms < best ? ms : best;
    }
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FLG_CUDA(cudaFreeAsync(sink, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    return FLG_OK;
}

}  // namespace flg

extern "C" int flg_measure_peaks(double *fp32_tflops, double *fp64_tflops, void *stream) {
    cudaStream_t st = flg::as_stream(stream);
    if (fp32_tflops) FLG_TRY(flg::time_fma<float>(40000, fp32_tflops, st));
    if (fp64_tflops) FLG_TRY(flg::time_fma<double>(2000, fp64_tflops, st));
    return FLG_OK;
}
