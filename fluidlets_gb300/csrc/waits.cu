// waits.cu -- flg_wait_selftest: the bounded device waits of waits.cuh driven to expiry.
//
// Each case launches a small kernel whose wait can never be satisfied, with a
// short limit, through the same wait functions the LU, the low-precision solve
// and the tensor-core update use.  The kernel must give up after the limit,
// raise its error word and return; the host then reads the word exactly as the
// production entry points do and returns their status for a wait that ran out
// (FLG_ERR_TIMEOUT), with the device still usable.  Nothing faults, traps or
// hangs: the waits end by themselves.
#include "flg_common.cuh"
#include "waits.cuh"

namespace flg {

struct SelftestWords {
    GridBar bar;       // the grid barrier: counter, error word
    unsigned slot[4];  // published values that nothing stores (preset to the unset pattern)
    int err;           // error word of the poll and mbarrier cases
};

// two CTAs wait at a grid barrier that expects three arrivals
__global__ void selftest_grid_kernel(SelftestWords *w, unsigned long long limit_ns) {
    grid_sync(&w->bar, gridDim.x + 1, limit_ns);
}

// one thread polls four values that nothing publishes
__global__ void selftest_poll_kernel(SelftestWords *w, unsigned long long limit_ns) {
    unsigned v[4] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu};
    wait_published4(w->slot, 4, 0xffffffffu, v, limit_ns, &w->err);
}

// one thread waits on an mbarrier phase that no arrival completes (the tensor-core
// update's ring waits), then on the same phase in draining mode
__global__ void selftest_mbar_kernel(SelftestWords *w, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && mbar_wait(&bar, 0, &w->err, limit_ns)) w->err = 2;  // 2: the wait succeeded
    __syncthreads();
}

}  // namespace flg

using namespace flg;

extern "C" size_t flg_wait_selftest_workspace(void) { return sizeof(SelftestWords) + 256; }

extern "C" int flg_wait_selftest(int which, double limit_ms, void *work, size_t work_bytes, void *stream) {
    FLG_REQUIRE(which >= 0 && which <= 2, "which must be 0 (grid barrier), 1 (published value) or 2 (mbarrier)");
    FLG_REQUIRE(limit_ms > 0.0 && limit_ms <= 10000.0, "limit must lie in (0, 10000] ms");
    Arena ar(work, work_bytes);
    SelftestWords *w = ar.take<SelftestWords>(1);
    FLG_REQUIRE(w != nullptr, "workspace too small for the wait self-test");
    cudaStream_t st = as_stream(stream);
    const unsigned long long limit_ns = (unsigned long long)(limit_ms * 1e6);
    FLG_CUDA(cudaMemsetAsync(w, 0, sizeof(SelftestWords), st));
    FLG_CUDA(cudaMemsetAsync(w->slot, 0xff, sizeof(w->slot), st));
    if (which == 0) {
        void *args[] = {&w, (void *)&limit_ns};
        FLG_CUDA(cudaLaunchCooperativeKernel((void *)selftest_grid_kernel, dim3(2), dim3(32), args, 0, st));
        count_launch();
    } else if (which == 1) {
        selftest_poll_kernel<<<1, 1, 0, st>>>(w, limit_ns);
        FLG_LAUNCH_CHECK();
    } else {
        selftest_mbar_kernel<<<1, 32, 0, st>>>(w, limit_ns);
        FLG_LAUNCH_CHECK();
    }
    SelftestWords h;
    FLG_CUDA(cudaMemcpyAsync(&h, w, sizeof(h), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    const int raised = which == 0 ? h.bar.err : h.err;
    if (raised == 1) {
        set_error("a bounded device wait timed out (self-test case %d)", which);
        return FLG_ERR_TIMEOUT;
    }
    return FLG_OK;  // the wait was satisfied, which the self-test's conditions rule out
}
