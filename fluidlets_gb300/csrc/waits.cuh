// waits.cuh -- the library's bounded device waits.
//
// Every spin-wait in a kernel of this library (the FP64 LU panel's grid
// barrier, the low-precision solve's dataflow polls, the tensor-core update's
// mbarrier waits) goes through one of the functions below.  Each takes a
// wall-clock limit in nanoseconds (the %globaltimer register, so the limit
// does not depend on the SM clock) and an error word: when the limit runs out
// the wait raises the word and returns false, and the kernel then skips its
// remaining work, drains its own asynchronous copies and returns, so the host
// reads an error status instead of the GPU hanging.  A wait also gives up as
// soon as another thread has raised the word.  flg_wait_selftest
// (waits.cu) drives each kind to expiry on a condition that nothing satisfies.
#pragma once
#include <stdint.h>

namespace flg {

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s per wait in production kernels

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed_u32(const void *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// ---- published-value poll ------------------------------------------------------------
// Waits until each of the `count` (<= 4) 32-bit words p[0..count) differs from `unset` (a
// producer stores the value itself, relaxed, in place of a flag).  v[] holds the caller's
// first probe of each word, so values that already arrived cost no extra load, and
// receives the values.  The words still unset are reloaded together on every round: values
// that arrive together cost one round trip, not one each.  The error word and the clock are
// checked every 32 rounds (all waiting threads share the error word).
__device__ __forceinline__ bool wait_published4(const unsigned *p, int count, unsigned unset, unsigned (&v)[4],
                                                unsigned long long limit_ns, int *err) {
    bool pending = false;
#pragma unroll
    for (int k = 0; k < 4; k++) pending |= k < count && v[k] == unset;
    if (!pending) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned round = 1;; round++) {
#pragma unroll
        for (int k = 0; k < 4; k++)
            if (k < count && v[k] == unset) v[k] = ld_relaxed_u32(p + k);
        pending = false;
#pragma unroll
        for (int k = 0; k < 4; k++) pending |= k < count && v[k] == unset;
        if (!pending) return true;
        if ((round & 31) == 0 && (*(volatile int *)err || global_ns() - t0 > limit_ns)) {
            atomicExch(err, 1);
            return false;
        }
    }
}

// ---- grid barrier -------------------------------------------------------------------
// One atomic per CTA: CTA 0 adds 2^31 - (nblocks - 1), every other CTA adds 1, so once
// all nblocks have arrived the counter has grown by exactly 2^31 and its top bit has
// flipped (no reset between barriers); waiters spin on an acquire load until it flips.
struct GridBar {
    unsigned int count;
    unsigned int pad;
    int err;   // a wait ran out
    int info;  // 1 + first zero pivot (the FP64 LU)
};

__device__ __forceinline__ bool grid_sync(GridBar *b, unsigned nblocks, unsigned long long limit_ns) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned inc = (blockIdx.x == 0) ? (0x80000000u - (nblocks - 1)) : 1u;
        unsigned old;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(&b->count), "r"(inc) : "memory");
        const unsigned long long t0 = global_ns();
        while (((old ^ ld_acquire_u32(&b->count)) & 0x80000000u) == 0) {
            if (*(volatile int *)&b->err || global_ns() - t0 > limit_ns) {
                atomicExch(&b->err, 1);
                break;
            }
        }
    }
    __syncthreads();
    return *(volatile int *)&b->err == 0;
}

// ---- mbarrier waits ---------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// false if the limit ran out (the error word is raised) or another role raised it
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (*(volatile int *)err) return false;
        if (global_ns() - t0 > limit_ns) {
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}
// the same, ignoring the error word: a role draining its own operations on the way out
__device__ __forceinline__ bool mbar_drain(uint64_t *bar, uint32_t parity, int *err, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (global_ns() - t0 > limit_ns) {
            atomicExch(err, 1);
            return false;
        }
    }
    return true;
}

}  // namespace flg
