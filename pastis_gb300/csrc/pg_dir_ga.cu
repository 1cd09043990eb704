// pg_dir_ga.cu -- the traceback-form DP and traceback kernels of
// X-drop (global alignment of each seed's region), in a translation unit of their own.
#include "pg_dir.h"

#include "pg_kernels_dir.cuh"

namespace pg {

cudaError_t dir_set_attributes_ga()
{
    const void *k[12] = {(const void *)k_ga_dir<0, false>, (const void *)k_ga_dir<1, false>,
                         (const void *)k_ga_dir<2, false>, (const void *)k_ga_dir<3, false>,
                         (const void *)k_ga_dir<0, true>, (const void *)k_ga_dir<1, true>,
                         (const void *)k_ga_dir<2, true>, (const void *)k_ga_dir<3, true>,
                         (const void *)k_ga_pair<0>, (const void *)k_ga_pair<1>,
                         (const void *)k_ga_pair<2>, (const void *)k_ga_pair<3>};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 12 && e == cudaSuccess; ++i)
        e = cudaFuncSetAttribute(k[i], cudaFuncAttributeMaxDynamicSharedMemorySize, DIR16_DYN_SMEM);
    return e;
}

template <bool CHK>
static void dp_ga(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
                   uint8_t *arena, int *dsc, int grid, int dyn, cudaStream_t st)
{
    const dim3 blk(WARPS * 32);
    switch (tie) {
    case 0: k_ga_dir<0, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 1: k_ga_dir<1, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 2: k_ga_dir<2, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    default: k_ga_dir<3, CHK><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    }
}

static void pair_ga(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
                    uint8_t *arena, int *dsc, int grid, int dyn, cudaStream_t st)
{
    const dim3 blk(WARPS * 32);
    switch (tie) {
    case 0: k_ga_pair<0><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 1: k_ga_pair<1><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    case 2: k_ga_pair<2><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    default: k_ga_pair<3><<<grid, blk, dyn, st>>>(kp, t0, t1, doff, arena, dsc); break;
    }
}

int dir_run_ga(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
               uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st)
{
    int launches = 2;
    dp_ga<false>(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, st);
    if (kp.dir16_pair) {
        cudaMemsetAsync(kp.counter, 0, sizeof(unsigned int), st);
        pair_ga(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, st);
        ++launches;
    }
    if (chk) {
        cudaMemsetAsync(kp.counter, 0, sizeof(unsigned int), st);
        dp_ga<true>(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, st);
        ++launches;
    }
    k_tb_ga<<<grid_tb, 256, 0, st>>>(kp, t0, t1, doff, arena, dsc);
    return launches;
}

}  // namespace pg
