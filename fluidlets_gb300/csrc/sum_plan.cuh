// sum_plan.cuh -- internal interface of the kernel-sum engine (sum.cu), used
// by the C-ABI entry point flg_evaluate and by the iterative solvers, which
// build the geometry part of a plan once and re-apply it to new strengths.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace flg {

// uniform cell list over the sources (device resident)
struct CellGrid {
    double ox, oy, oz, h, inv_h;
    int nx, ny, nz, ncell;
};

struct SumLayout {
    int nf;    // strength vectors per source: 1 real, 2 complex
    bool ck;   // complex kernel (complex Brinkman alpha)
    int outw;  // accumulator width per target (3 or 6)
    int NQ;    // float4 slots per packed source
    int64_t S, split_len;  // source splits over gridDim.y
};

// device buffers carved from the caller's workspace
struct SumPlan {
    double *partial;  // [S][M][outw], target in processing order
    float4 *packed;   // [N][NQ] FP32 sources in cell order (mixed only)
    float4 *tile_box; // [ceil(N / 256)][2]: lo x, y, z, max threshold | hi x, y, z
    CellGrid *grid;
    double *bounds;
    int *cell_of, *counts, *offsets, *block_sums, *sorted;
    int *tcell, *toffsets, *tperm;  // targets bucketed by source cell (large target sets)
};

struct SumRun {
    int kind;
    const double *tg;
    int64_t M;
    const double *src, *eps, *f;
    int64_t N;
    double alpha_re, alpha_im, mu_re, mu_im;
    double *out;
    int out_complex;
};

int check_kernel_args(int kind, double alpha_re, double alpha_im);
void sum_layout(int kind, int64_t M, int64_t N, int nf, bool ck, int precision, SumLayout &L);
size_t sum_workspace_bytes(int kind, int64_t M, int64_t N, int nf, bool ck, int precision);
int sum_plan_carve(void *work, size_t work_bytes, int64_t M, int64_t N, const SumLayout &L, int precision,
                   SumPlan *p);
int sum_plan_geometry(const double *src, const double *eps, int64_t N, const SumLayout &L, SumPlan *p,
                      cudaStream_t st);
int sum_run(const SumRun &r, const SumLayout &L, int precision, const SumPlan *p, cudaStream_t st);

}  // namespace flg
