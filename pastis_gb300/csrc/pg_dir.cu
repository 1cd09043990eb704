// pg_dir.cu -- the traceback form of the alignment DP: the sizing and chunk
// kernels and the launchers (pg_dir.h).  The DP and traceback kernels of the
// two modes compile in translation units of their own (pg_dir_ga.cu,
// pg_dir_sw.cu), in parallel with the rest.
#include "pg_dir.h"

#include "pg_kernels_dir.cuh"

namespace pg {

cudaError_t dir_set_attributes()
{
    const cudaError_t e = dir_set_attributes_ga();
    return e != cudaSuccess ? e : dir_set_attributes_sw();
}

void dir_sizes(bool xdrop, const KParams &kp, uint64_t *bytes, unsigned long long *nchk, int grid,
               cudaStream_t st)
{
    if (xdrop) k_dirsize<true><<<grid, 256, 0, st>>>(kp, bytes, nchk);
    else k_dirsize<false><<<grid, 256, 0, st>>>(kp, bytes, nchk);
}

void dir_chunk_end(const uint64_t *doff, uint64_t t0, uint64_t n, uint64_t budget, uint64_t *t1,
                   cudaStream_t st)
{
    k_chunk_end<<<1, 32, 0, st>>>(doff, t0, n, budget, t1);
}

int dir_run(bool xdrop, int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
            uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st)
{
    return xdrop ? dir_run_ga(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, grid_tb, chk, st)
                 : dir_run_sw(tie, kp, t0, t1, doff, arena, dsc, grid, dyn, grid_tb, chk, st);
}

}  // namespace pg
