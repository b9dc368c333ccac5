// flg_common.cuh -- shared definitions of libfluidlets_gb300 (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "../../include/fluidlets_gb300.h"

namespace flg {

constexpr double kPi = 3.141592653589793;
constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs (queried at run time where it matters)

// Thread-local text of the last failure, returned by flg_last_error().
void set_error(const char *fmt, ...);

// Host-side argument check: records the message and returns FLG_ERR_INVALID.
#define FLG_REQUIRE(cond, ...)                 \
    do {                                       \
        if (!(cond)) {                         \
            ::flg::set_error(__VA_ARGS__);     \
            return FLG_ERR_INVALID;            \
        }                                      \
    } while (0)

#define FLG_CUDA(call)                                                                      \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) {                                                            \
            ::flg::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return FLG_ERR_CUDA;                                                            \
        }                                                                                   \
    } while (0)

// every launch site of the library ends with FLG_LAUNCH_CHECK(): it counts
// the launch (flg_launch_count) and turns a launch error into FLG_ERR_CUDA
void count_launch();
#define FLG_LAUNCH_CHECK()            \
    do {                              \
        ::flg::count_launch();        \
        FLG_CUDA(cudaGetLastError()); \
    } while (0)

// CUDA-event timing of profiled kernels (flg_profile_enable)
void prof_begin(int slot, cudaStream_t st);
void prof_end(int slot, cudaStream_t st);
// scope in which this thread's launches record no timing events (graph capture)
struct ProfSuppress {
    ProfSuppress();
    ~ProfSuppress();
};

#define FLG_TRY(call)            \
    do {                         \
        int s_ = (call);         \
        if (s_ != FLG_OK) return s_; \
    } while (0)

inline int sm_count() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = kNumSMs;
    }
    return n;
}

// Bump allocator over a caller-provided workspace (256-byte aligned slices).
struct Arena {
    char *base;
    size_t cap, used;
    Arena(void *p, size_t n) : base((char *)p), cap(n), used(0) {}
    template <typename T>
    T *take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        size_t bytes = count * sizeof(T);
        if (off + bytes > cap || (base == nullptr && bytes > 0)) return nullptr;
        used = off + bytes;
        return (T *)(base + off);
    }
};

// Byte counter with Arena's interface, for *_workspace() queries: the same
// carving code runs once against each, so sizes and offsets always agree.
struct CountingArena {
    size_t used = 0;
    template <typename T>
    T *take(size_t count) {
        used = ((used + 255) & ~size_t(255)) + count * sizeof(T);
        return nullptr;
    }
    size_t bytes() const { return used + 256; }
};

inline cudaStream_t as_stream(void *s) { return (cudaStream_t)s; }

// NVTX range around a C-ABI entry point (a profiler shows the library's calls on the host
// timeline; without a tool attached a push/pop costs a few nanoseconds)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};
#define FLG_RANGE(name) ::flg::NvtxRange flg_nvtx_range_(name)

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// the same tensor-core update applied to `count` independent systems: C, Lp and Ut of
// system z at + z * (sC, sL, sU) elements (tc_gemm.cu)
struct TcBatch {
    int count = 1;
    int64_t sC = 0, sL = 0, sU = 0;
};

}  // namespace flg
