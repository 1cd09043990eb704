// pg_stat.cu -- the statistics form of the alignment DP (k_ga / k_sw: the
// statistics words ride along the DP, no traceback) in a translation unit of
// its own, compiled in parallel with the others; launchers in pg_stat.h.
#include "pg_stat.h"

namespace pg {

cudaError_t stat_set_attributes()
{
    const void *k[8] = {(const void *)k_ga<0>, (const void *)k_ga<1>, (const void *)k_ga<2>,
                        (const void *)k_ga<3>, (const void *)k_sw<0>, (const void *)k_sw<1>,
                        (const void *)k_sw<2>, (const void *)k_sw<3>};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 8 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, DP_DYN_SMEM);
    return e;
}

cudaError_t stat_occupancy(bool xdrop, int *per_sm)
{
    return xdrop ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_ga<0>, WARPS * 32, DP_DYN_SMEM)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_sw<0>, WARPS * 32, DP_DYN_SMEM);
}

void stat_run(bool xdrop, int tie, const KParams &kp, int grid, int dyn, cudaStream_t st)
{
    const dim3 blk(WARPS * 32);
    if (xdrop) {
        switch (tie) {
        case 0: k_ga<0><<<grid, blk, dyn, st>>>(kp); break;
        case 1: k_ga<1><<<grid, blk, dyn, st>>>(kp); break;
        case 2: k_ga<2><<<grid, blk, dyn, st>>>(kp); break;
        default: k_ga<3><<<grid, blk, dyn, st>>>(kp); break;
        }
    } else {
        switch (tie) {
        case 0: k_sw<0><<<grid, blk, dyn, st>>>(kp); break;
        case 1: k_sw<1><<<grid, blk, dyn, st>>>(kp); break;
        case 2: k_sw<2><<<grid, blk, dyn, st>>>(kp); break;
        default: k_sw<3><<<grid, blk, dyn, st>>>(kp); break;
        }
    }
}

}  // namespace pg
