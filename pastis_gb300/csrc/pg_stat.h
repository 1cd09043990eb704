// pg_stat.h -- host launchers of the statistics form of the alignment DP,
// k_ga / k_sw (pg_kernels.cuh, compiled in pg_stat.cu).
#pragma once
#include <cuda_runtime.h>

#include "pg_kernels.cuh"

namespace pg {

// lets k_ga / k_sw take DP_DYN_SMEM of dynamic shared memory
cudaError_t stat_set_attributes();
// resident blocks per SM of k_ga (xdrop) or k_sw
cudaError_t stat_occupancy(bool xdrop, int *per_sm);
// one launch over the batch: grid blocks, dyn bytes of dynamic shared memory
void stat_run(bool xdrop, int tie, const KParams &kp, int grid, int dyn, cudaStream_t st);

}  // namespace pg
