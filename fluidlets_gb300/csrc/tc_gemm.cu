// tc_gemm.cu -- tcgen05 tensor-core rank-K update for the low-precision LU.
//
//   C (m x nc, FP32, row-major, ldc)  -=  A (m x K) * B^T,  B given as Bt (nc x K)
//   (or, in store mode, C = A * B^T)
//
// Both operands are K-major (K contiguous per row, K a multiple of 128).  A
// batch of equally shaped updates of independent systems (fixed strides
// between their C, A and Bt) is one launch: the tensor maps are 3-D, the
// system index their outer coordinate.  A persistent kernel, one CTA per SM
// (the caller may cap the grid below the SM count), walks the 128 x BN tiles
// of C over all systems (BN = 256, or 128 for narrow or small updates, chosen
// per call):
//   * warp 0 (one lane) streams K-blocks of A and B (128 B = 32 TF32 or 64 BF16
//     per row) with TMA (cp.async.bulk.tensor, 128-byte swizzle) into a
//     shared-memory ring guarded by mbarriers (4 stages at BN = 256, 6 at 128);
//   * warp 1 (one lane) issues tcgen05.mma (cta_group::1, M = 128, N = BN;
//     kind::tf32, or kind::f16 with BF16 operands) into one of two BN-column
//     TMEM accumulators and releases each stage with tcgen05.commit;
//   * warps 2-5 drain the other accumulator (tcgen05.ld, 32 TMEM lanes each),
//     stage -acc in 32 x 32 swizzled boxes and add them to C with TMA
//     reduce-add (cp.reduce.async.bulk.tensor): C is never read by the SM and
//     the epilogue of one tile overlaps the MMAs of the next.
// Every mbarrier wait is bounded; on a timeout the kernel raises an error
// flag, skips the remaining work, waits (bounded) for its own TMA loads and
// MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>

#include "flg_common.cuh"
#include "waits.cuh"

namespace flg {

constexpr int TC_BM = 128, TC_THREADS = 192, TC_EPI_WARPS = 4;
constexpr int TC_A_BYTES = TC_BM * 128;   // A tile of a K-block: 128 rows x 128 B
constexpr int TC_STG_BYTES = 32 * 128;    // one 32 x 32 FP32 staging box

// tile width BN: ring depth, B tile bytes (BN rows x 128 B), TMEM columns (two accumulators)
template <int BN>
struct TcTile {
    static_assert(BN == 128 || BN == 256, "tile width");
    static constexpr int STAGES = BN == 256 ? 4 : 6;
    static constexpr int B_BYTES = BN * 128;
    static constexpr uint32_t TMEM_COLS = 2 * BN;
    static constexpr size_t SMEM = 1024 + STAGES * (TC_A_BYTES + B_BYTES) + TC_EPI_WARPS * 2 * TC_STG_BYTES;
    static_assert(SMEM <= 232448 - 256, "shared memory per CTA");
};

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 3-D tiles: x (innermost, 16-byte aligned), row y, system z
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], "
        "[%2];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int x, int y, int z) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
                     (uint64_t)map),
                 "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
                 : "memory");
}
__device__ __forceinline__ void tma_reduce_add_3d(const CUtensorMap *map, const void *src, int x, int y, int z) {
    asm volatile(
        "cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(
            (uint64_t)map),
        "r"(smem_u32(src)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(const void *p) {
    const uint64_t addr = smem_u32(p);
    uint64_t d = 0;
    d |= (addr >> 4) & 0x3FFFull;            // start address
    d |= (uint64_t)1 << 16;                  // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;        // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                  // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                  // swizzle mode: 128B
    return d;
}

// instruction descriptor: D = F32, A/B format (TF32 = 2, BF16 = 1), K-major A and B, M = 128, N = bn
__host__ __device__ constexpr uint32_t tc_idesc(uint32_t fmt, int bn) {
    return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(bn >> 3) << 17) | ((uint32_t)(TC_BM >> 4) << 24);
}

template <int MODE, int TC_BN>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_update_kernel(const __grid_constant__ CUtensorMap tmA,
                                                                  const __grid_constant__ CUtensorMap tmB,
                                                                  const __grid_constant__ CUtensorMap tmC, int m,
                                                                  int nc, int nkb, int nbat, int store, int *err) {
    constexpr int KBLK = MODE == FLG_LU_TF32 ? 32 : 64;  // elements per 128-byte row
    constexpr int KSTEP_BYTES = 32;                       // one MMA consumes 32 bytes of each row
    constexpr uint32_t IDESC = tc_idesc(MODE == FLG_LU_TF32 ? 2u : 1u, TC_BN);
    constexpr int TC_STAGES = TcTile<TC_BN>::STAGES, TC_B_BYTES = TcTile<TC_BN>::B_BYTES;
    constexpr uint32_t TC_TMEM_COLS = TcTile<TC_BN>::TMEM_COLS;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem, *sB = smem + TC_STAGES * TC_A_BYTES, *stg = sB + TC_STAGES * TC_B_BYTES;
    __shared__ __align__(8) uint64_t full[TC_STAGES], empty[TC_STAGES], accf[2], acce[2], mma_done;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // tile t: system t / (ntx nty), then row block, then column block
    const int ntx = (nc + TC_BN - 1) / TC_BN, nty = (m + TC_BM - 1) / TC_BM, nper = ntx * nty, ntiles = nper * nbat;

    if (threadIdx.x == 0) {
        for (int s = 0; s < TC_STAGES; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], TC_EPI_WARPS);
        }
        mbar_init(&mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(TC_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (warp == 0) {
        if (lane == 0) {  // TMA producer: global K-block counter g -> stage g % S, use g / S
            uint32_t g = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int z = t / nper, tr = t - z * nper, m0 = (tr / ntx) * TC_BM, n0 = (tr % ntx) * TC_BN;
                for (int kb = 0; kb < nkb; kb++, g++) {
                    const int s = g % TC_STAGES;
                    const uint32_t use = g / TC_STAGES;
                    if (use > 0 && !mbar_wait(&empty[s], (use & 1) ^ 1, err, kWaitLimitNs)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&full[s], TC_A_BYTES + TC_B_BYTES);
                    tma_load_3d(sA + s * TC_A_BYTES, &tmA, &full[s], kb * KBLK, m0, z);
                    tma_load_3d(sB + s * TC_B_BYTES, &tmB, &full[s], kb * KBLK, n0, z);
                }
            }
            // the last (up to S) loads issued must have landed before the CTA exits
            for (uint32_t q = (g > TC_STAGES ? g - TC_STAGES : 0); q < g; q++)
                mbar_drain(&full[q % TC_STAGES], (q / TC_STAGES) & 1, err, kWaitLimitNs);
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            uint32_t g = 0, i = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, i++) {
                const uint32_t buf = i & 1, ause = i >> 1;
                if (ause > 0 && !mbar_wait(&acce[buf], (ause & 1) ^ 1, err, kWaitLimitNs)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t d = tmem + buf * TC_BN;
                for (int kb = 0; kb < nkb; kb++, g++) {
                    const int s = g % TC_STAGES;
                    const uint32_t use = g / TC_STAGES;
                    if (!mbar_wait(&full[s], use & 1, err, kWaitLimitNs)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                    for (int kk = 0; kk < 128 / KSTEP_BYTES; kk++) {
                        const uint64_t ad = sw128_desc(sA + s * TC_A_BYTES + kk * KSTEP_BYTES);
                        const uint64_t bd = sw128_desc(sB + s * TC_B_BYTES + kk * KSTEP_BYTES);
                        const uint32_t acc = (kb | kk) ? 1u : 0u;
                        if constexpr (MODE == FLG_LU_TF32) {
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                                : "memory");
                        } else {
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d),
                                "l"(ad), "l"(bd), "r"(IDESC), "r"(acc)
                                : "memory");
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_u32(&empty[s]))
                                 : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&accf[buf]))
                             : "memory");
            }
            // every MMA issued has completed before the TMEM is freed
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&mma_done))
                         : "memory");
            mbar_drain(&mma_done, 0, err, kWaitLimitNs);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +32, i.e. tile rows 32 (w % 4) + lane
        const int q = warp & 3;
        uint8_t *mystg = stg + (warp - 2) * 2 * TC_STG_BYTES;
        uint32_t i = 0, nst = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, i++) {
            const uint32_t buf = i & 1, ause = i >> 1;
            // warp-uniform: tcgen05.ld.sync.aligned must be executed by the whole warp
            if (!__all_sync(0xffffffffu, mbar_wait(&accf[buf], ause & 1, err, kWaitLimitNs))) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int z = t / nper, tr = t - z * nper, m0 = (tr / ntx) * TC_BM, n0 = (tr % ntx) * TC_BN;
#pragma unroll 1
            for (int ch = 0; ch < TC_BN / 32; ch++, nst++) {
                uint32_t v[32];
                const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + buf * TC_BN + (uint32_t)(ch * 32);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
                    "[%32];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                      "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                      "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                // staging box nst % 2: the reduce that last read it (two boxes ago) must be done
                uint8_t *box = mystg + (nst & 1) * TC_STG_BYTES;
                if (nst >= 2 && lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                __syncwarp();
                // row `lane`, 16-byte chunk c at chunk position c ^ (row % 8) (128-byte swizzle)
                const float sg = store ? 1.0f : -1.0f;  // C = acc, or C += -acc
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const float4 w = make_float4(sg * __uint_as_float(v[4 * c]), sg * __uint_as_float(v[4 * c + 1]),
                                                 sg * __uint_as_float(v[4 * c + 2]), sg * __uint_as_float(v[4 * c + 3]));
                    *reinterpret_cast<float4 *>(box + lane * 128 + ((c ^ (lane & 7)) << 4)) = w;
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) {
                    if (store) tma_store_3d(&tmC, box, n0 + ch * 32, m0 + q * 32, z);
                    else tma_reduce_add_3d(&tmC, box, n0 + ch * 32, m0 + q * 32, z);
                    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                }
            }
            // this accumulator's TMEM reads are complete: hand it back to the MMA issuer
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acce[buf]);
        }
        if (lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        __syncwarp();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS)
                     : "memory");
}

// system blockIdx.y: src + y ss (rows x K, row stride lds) -> dst + y rows K (compact)
__global__ void f32_to_bf16_rows_kernel(const float *src, int64_t lds, int64_t ss, __nv_bfloat16 *dst, int64_t rows,
                                        int64_t K) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * K) return;
    const int64_t r = i / K, k = i % K;
    dst[blockIdx.y * rows * K + i] = __float2bfloat16_rn(src[blockIdx.y * ss + r * lds + k]);
}

// ---- host side ---------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// the stride between systems of a batch in bytes (one system: the matrix's own extent)
static int64_t system_stride_bytes(int nb, int64_t stride_elems, int64_t rows, int64_t ld_elems, size_t esz) {
    return (int64_t)esz * (nb > 1 ? stride_elems : std::max<int64_t>(rows, 1) * ld_elems);
}

// operand map: nb systems (stride sb elements) of rows x K K-major elements (row stride
// ld_elems), box box_rows x 128 bytes x 1 system, 128B swizzle
static int make_operand_map(CUtensorMap *map, const void *base, int64_t rows, int64_t K, int64_t ld_elems, int mode,
                            int box_rows, int nb = 1, int64_t sb = 0) {
    auto fn = encode_fn();
    FLG_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled unavailable");
    const bool bf = mode == FLG_LU_BF16;
    const size_t esz = bf ? 2 : 4;
    const int64_t sbb = system_stride_bytes(nb, sb, rows, ld_elems, esz);
    FLG_REQUIRE(((uintptr_t)base & 15) == 0 && (ld_elems * esz) % 16 == 0 && sbb % 16 == 0,
                "TMA operand not 16-byte aligned");
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)nb};
    cuuint64_t strides[2] = {(cuuint64_t)(ld_elems * esz), (cuuint64_t)sbb};
    cuuint32_t box[3] = {(cuuint32_t)(128 / esz), (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, bf ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                    const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FLG_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FLG_OK;
}

// C map: nb systems (stride sb elements) of m x nc FP32 (row stride ldc), 32 x 32 x 1 boxes,
// 128B swizzle (the epilogue's staging layout)
static int make_c_map(CUtensorMap *map, float *C, int64_t m, int64_t nc, int64_t ldc, int nb = 1, int64_t sb = 0) {
    auto fn = encode_fn();
    FLG_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled unavailable");
    const int64_t sbb = system_stride_bytes(nb, sb, m, ldc, 4);
    FLG_REQUIRE(((uintptr_t)C & 15) == 0 && (ldc * 4) % 16 == 0 && sbb % 16 == 0, "C not 16-byte aligned");
    cuuint64_t dims[3] = {(cuuint64_t)nc, (cuuint64_t)m, (cuuint64_t)nb};
    cuuint64_t strides[2] = {(cuuint64_t)(ldc * 4), (cuuint64_t)sbb};
    cuuint32_t box[3] = {32, 32, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, C, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FLG_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed for C (%d)", (int)r);
    return FLG_OK;
}

// plain FP32 box map (no swizzle): rows x cols, row stride ld elements, boxes of
// box_rows x box_cols; reads outside the matrix return zeros
int make_box_map_f32(CUtensorMap *map, const float *base, int64_t rows, int64_t cols, int64_t ld, int box_rows,
                     int box_cols) {
    auto fn = encode_fn();
    FLG_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled unavailable");
    FLG_REQUIRE(((uintptr_t)base & 15) == 0 && (ld * 4) % 16 == 0 && (box_cols * 4) % 16 == 0,
                "TMA box map not 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    FLG_REQUIRE(r == CUDA_SUCCESS, "cuTensorMapEncodeTiled failed for a box map (%d)", (int)r);
    return FLG_OK;
}

static int sm_count_of_current_device() {
    static std::mutex mu;
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    std::lock_guard<std::mutex> lock(mu);
    if (!cached[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 148;
    }
    return cached[dev];
}

size_t tc_update_bytes(int64_t m, int64_t nc, int64_t K, int mode, int nb) {
    CountingArena c;
    c.take<int>(1);
    if (mode == FLG_LU_BF16) {
        c.take<__nv_bfloat16>((size_t)nb * m * K);
        c.take<__nv_bfloat16>((size_t)nb * nc * K);
    }
    return c.bytes();
}

// Tile width for an m x nc update: the one whose waves over the SMs take the
// least time, a 128 x BN tile costing about (128 + BN) units (operand bytes per
// K-block).  BN = 256 reads 25 % fewer operand bytes per output; BN = 128 gives
// twice the tiles for small updates and wastes nothing on updates of 128 columns.
int tc_pick_tile(int64_t m, int64_t nc, int sms, int nb = 1) {
    const int64_t ty = nb * ceil_div(m, TC_BM);
    const int64_t w256 = ceil_div(ty * ceil_div(nc, 256), sms), w128 = ceil_div(ty * ceil_div(nc, 128), sms);
    return w128 * (128 + 128) < w256 * (128 + 256) ? 128 : 256;
}

template <int MODE, int BN>
static int tc_launch(const CUtensorMap &ma, const CUtensorMap &mb, const CUtensorMap &mc, int64_t m, int64_t nc,
                     int nkb, int nb, bool store, int *err, int sms, cudaStream_t st) {
    static bool attr_set = false;  // set once, so a later call can be captured in a graph
    if (!attr_set) {
        FLG_CUDA(cudaFuncSetAttribute(tc_update_kernel<MODE, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)TcTile<BN>::SMEM));
        attr_set = true;
    }
    const int64_t ntiles = nb * ceil_div(m, TC_BM) * ceil_div(nc, BN);
    FLG_REQUIRE(ntiles < (1LL << 31), "too many tiles");
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, sms);
    tc_update_kernel<MODE, BN><<<grid, TC_THREADS, TcTile<BN>::SMEM, st>>>(ma, mb, mc, (int)m, (int)nc, nkb, nb,
                                                                           store ? 1 : 0, err);
    FLG_LAUNCH_CHECK();
    return FLG_OK;
}

// The launch and the timeout check shared by both entry points below: C map, grid, flag.
static int tc_run(const CUtensorMap &ma, const CUtensorMap &mb, float *C, int64_t ldc, int64_t m, int64_t nc,
                  int64_t K, int mode, int bn, int sms, const TcBatch &bt, bool store, int *err, bool own_err,
                  cudaStream_t st) {
    const int nb = bt.count;
    CUtensorMap mc;
    FLG_TRY(make_c_map(&mc, C, m, nc, ldc, nb, bt.sC));
    if (own_err) FLG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    const int nkb = (int)(K / (mode == FLG_LU_TF32 ? 32 : 64));
    int rc;
    if (mode == FLG_LU_TF32)
        rc = bn == 128 ? tc_launch<FLG_LU_TF32, 128>(ma, mb, mc, m, nc, nkb, nb, store, err, sms, st)
                       : tc_launch<FLG_LU_TF32, 256>(ma, mb, mc, m, nc, nkb, nb, store, err, sms, st);
    else
        rc = bn == 128 ? tc_launch<FLG_LU_BF16, 128>(ma, mb, mc, m, nc, nkb, nb, store, err, sms, st)
                       : tc_launch<FLG_LU_BF16, 256>(ma, mb, mc, m, nc, nkb, nb, store, err, sms, st);
    FLG_TRY(rc);
    if (!own_err) return FLG_OK;
    int herr = 0;
    FLG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FLG_CUDA(cudaStreamSynchronize(st));
    if (herr != 0) {
        set_error("a bounded device wait timed out (tensor-core update, mbarrier)");
        return FLG_ERR_TIMEOUT;
    }
    return FLG_OK;
}

static int tc_check_shape(int64_t m, int64_t nc, int64_t K, int tile, const TcBatch &bt) {
    FLG_REQUIRE(m >= 0 && nc >= 0 && m < (1LL << 31) && nc < (1LL << 31), "bad tensor-core update shape");
    FLG_REQUIRE(bt.count >= 1 && bt.count <= 65535, "bad batch count %d", bt.count);
    FLG_REQUIRE(K > 0 && K % 128 == 0 && K <= (1 << 20), "tensor-core update depth must be a multiple of 128");
    FLG_REQUIRE(tile == 0 || tile == 128 || tile == 256, "tile width must be 128 or 256 (or 0 to choose)");
    return FLG_OK;
}

// err_dev: device flag raised on a timed-out wait.  When null, the flag lives in
// the workspace and the call synchronizes to check it; the LU passes its own
// flag and checks it once at the end of the factorization.  tile: 0 picks the
// tile width (tc_pick_tile), 128 or 256 forces it.  max_ctas > 0 caps the
// persistent grid (leaving SMs to work on another stream).  bt: the same update
// of bt.count systems, C, Lp and Ut of system z at + z * (bt.sC, bt.sL, bt.sU).
int tc_update(float *C, int64_t ldc, const float *Lp, int64_t ldl, const float *Ut, int64_t ldu, int64_t m,
              int64_t nc, int64_t K, int mode, void *work, size_t work_bytes, cudaStream_t st, int *err_dev,
              bool store, int tile, int max_ctas, const TcBatch &bt) {
    FLG_REQUIRE(mode == FLG_LU_TF32 || mode == FLG_LU_BF16, "tensor-core mode must be TF32 or BF16");
    FLG_TRY(tc_check_shape(m, nc, K, tile, bt));
    const int nb = bt.count;
    if (m == 0 || nc == 0) return FLG_OK;
    const int sms = max_ctas > 0 ? std::min(max_ctas, sm_count_of_current_device()) : sm_count_of_current_device();
    const int bn = tile ? tile : tc_pick_tile(m, nc, sms, nb);
    Arena ar(work, work_bytes);
    int *own = ar.take<int>(1);
    int *err = err_dev ? err_dev : own;
    FLG_REQUIRE(err != nullptr && own != nullptr, "workspace too small for the tensor-core update");
    CUtensorMap ma, mb;
    if (mode == FLG_LU_TF32) {
        FLG_TRY(make_operand_map(&ma, Lp, m, K, ldl, mode, TC_BM, nb, bt.sL));
        FLG_TRY(make_operand_map(&mb, Ut, nc, K, ldu, mode, bn, nb, bt.sU));
    } else {
        __nv_bfloat16 *La = ar.take<__nv_bfloat16>((size_t)nb * m * K);
        __nv_bfloat16 *Ub = ar.take<__nv_bfloat16>((size_t)nb * nc * K);
        FLG_REQUIRE(La && Ub, "workspace too small for the BF16 operands");
        f32_to_bf16_rows_kernel<<<dim3((unsigned)ceil_div(m * K, 256), nb), 256, 0, st>>>(Lp, ldl, bt.sL, La, m, K);
        FLG_LAUNCH_CHECK();
        f32_to_bf16_rows_kernel<<<dim3((unsigned)ceil_div(nc * K, 256), nb), 256, 0, st>>>(Ut, ldu, bt.sU, Ub, nc,
                                                                                             K);
        FLG_LAUNCH_CHECK();
        FLG_TRY(make_operand_map(&ma, La, m, K, K, mode, TC_BM, nb, m * K));
        FLG_TRY(make_operand_map(&mb, Ub, nc, K, K, mode, bn, nb, nc * K));
    }
    return tc_run(ma, mb, C, ldc, m, nc, K, mode, bn, sms, bt, store, err, err_dev == nullptr, st);
}

// The BF16 update with operands already rounded to BF16 (K-major, row strides ldl / ldu
// elements, system strides bt.sL / bt.sU elements): no conversion launches.  C -= La Ub^T.
int tc_update_bf16(float *C, int64_t ldc, const void *La, int64_t ldl, const void *Ub, int64_t ldu, int64_t m,
                   int64_t nc, int64_t K, void *work, size_t work_bytes, cudaStream_t st, int *err_dev, int tile,
                   int max_ctas, const TcBatch &bt) {
    FLG_TRY(tc_check_shape(m, nc, K, tile, bt));
    const int nb = bt.count;
    if (m == 0 || nc == 0) return FLG_OK;
    const int sms = max_ctas > 0 ? std::min(max_ctas, sm_count_of_current_device()) : sm_count_of_current_device();
    const int bn = tile ? tile : tc_pick_tile(m, nc, sms, nb);
    Arena ar(work, work_bytes);
    int *own = ar.take<int>(1);
    int *err = err_dev ? err_dev : own;
    FLG_REQUIRE(err != nullptr && own != nullptr, "workspace too small for the tensor-core update");
    CUtensorMap ma, mb;
    FLG_TRY(make_operand_map(&ma, La, m, K, ldl, FLG_LU_BF16, TC_BM, nb, bt.sL));
    FLG_TRY(make_operand_map(&mb, Ub, nc, K, ldu, FLG_LU_BF16, bn, nb, bt.sU));
    return tc_run(ma, mb, C, ldc, m, nc, K, FLG_LU_BF16, bn, sms, bt, false, err, err_dev == nullptr, st);
}

}  // namespace flg

extern "C" size_t flg_tc_rank_update_workspace(int64_t m, int64_t nc, int mode) {
    return flg::tc_update_bytes(m, nc, 128, mode, 1);
}

extern "C" int flg_tc_rank_update(float *C, int64_t ldc, const float *A, int64_t lda, const float *Bt, int64_t ldb,
                                  int64_t m, int64_t nc, int mode, void *work, size_t work_bytes, void *stream) {
    FLG_RANGE("flg_tc_rank_update");
    FLG_REQUIRE(ldb == 128, "Bt must be compact (ldb == 128)");
    FLG_REQUIRE(lda >= 128 && ldc >= nc, "bad leading dimensions");
    return flg::tc_update(C, ldc, A, lda, Bt, 128, m, nc, 128, mode, work, work_bytes, flg::as_stream(stream), nullptr,
                          false, 0, 0, flg::TcBatch{});
}
