// pg_dir_sw.cu -- the traceback-form DP and traceback kernels of
// Smith-Waterman (local alignment), in a translation unit of their own.
#include "pg_dir.h"

#include "pg_kernels_dir.cuh"

namespace pg {

cudaError_t dir_set_attributes_sw()
{
    const void *k[8] = {(const void *)k_sw_dir<0, false>, (const void *)k_sw_dir<1, false>,
                        (const void *)k_sw_dir<2, false>, (const void *)k_sw_dir<3, false>,
                        (const void *)k_sw_dir<0, true>, (const void *)k_sw_dir<1, true>,
                        (const void *)k_sw_dir<2, true>, (const void *)k_sw_dir<3, true>};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 8 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, DIR16_DYN_SMEM);
    return e;
}

template <bool CHK>
static void dp_sw(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
                   uint8_t *arena, int *dsc, int grid, int dyn, cudaStream_t st)
{
    const dim3 blk(WARPS * 32);
    switch (tie) {
    case 0: k_sw_dir<0, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 1: k_sw_dir<1, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 2: k_sw_dir<2, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    default: k_sw_dir<3, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    }
}

int dir_run_sw(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
               uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st)
{
    int launches = 2;
    dp_sw<false>(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, st);   // with the half-warp pairs
    if (chk) {
        cudaMemsetAsync(kp.counter, 0, sizeof(unsigned int), st);
        dp_sw<true>(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, st);
        ++launches;
    }
    k_tb_sw<<<grid_tb, 256, 0, st>>>(kp, t0, t1, doff, arena, dsc);
    return launches;
}

}  // namespace pg
