// pg_dir.cu -- the traceback form of the alignment DP in a translation unit
// of its own (its 32 DP instantiations per tie policy compile in parallel
// with pg_api.cu); launchers declared in pg_dir.h.
#include "pg_dir.h"

#include "pg_kernels_dir.cuh"

namespace pg {

cudaError_t dir_set_attributes()
{
    const int b = DIR16_DYN_SMEM;
    cudaError_t e = cudaSuccess;
    const void *k[8] = {(const void *)k_ga_dir<0>, (const void *)k_ga_dir<1>, (const void *)k_ga_dir<2>,
                        (const void *)k_ga_dir<3>, (const void *)k_sw_dir<0>, (const void *)k_sw_dir<1>,
                        (const void *)k_sw_dir<2>, (const void *)k_sw_dir<3>};
    for (int i = 0; i < 8 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return e;
}

void dir_sizes(bool xdrop, const KParams &kp, uint64_t *bytes, int grid, cudaStream_t st)
{
    if (xdrop) k_dirsize<true><<<grid, 256, 0, st>>>(kp, bytes);
    else k_dirsize<false><<<grid, 256, 0, st>>>(kp, bytes);
}

void dir_chunk_end(const uint64_t *doff, uint64_t t0, uint64_t n, uint64_t budget, uint64_t *t1,
                   cudaStream_t st)
{
    k_chunk_end<<<1, 32, 0, st>>>(doff, t0, n, budget, t1);
}

void dir_run(bool xdrop, int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
             uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, cudaStream_t st)
{
    const dim3 blk(WARPS * 32);
    if (xdrop) {
        switch (tie) {
        case 0: k_ga_dir<0><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        case 1: k_ga_dir<1><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        case 2: k_ga_dir<2><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        default: k_ga_dir<3><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        }
        k_tb_ga<<<grid_tb, 256, 0, st>>>(kp, t0, t1, doff, arena, dsc);
    } else {
        switch (tie) {
        case 0: k_sw_dir<0><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        case 1: k_sw_dir<1><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        case 2: k_sw_dir<2><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        default: k_sw_dir<3><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
        }
        k_tb_sw<<<grid_tb, 256, 0, st>>>(kp, t0, t1, doff, arena, dsc);
    }
}

}  // namespace pg
