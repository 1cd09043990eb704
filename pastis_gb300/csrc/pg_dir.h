// pg_dir.h -- host launchers of the traceback form of the alignment DP
// (kernels in pg_kernels_dir.cuh, compiled in pg_dir.cu, pg_dir_ga.cu and
// pg_dir_sw.cu).  All launches go to
// stream st; errors surface through cudaGetLastError.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "pg_kernels.cuh"

namespace pg {

// lets k_ga_dir / k_ga_pair / k_sw_dir take DIR16_DYN_SMEM of dynamic shared memory
cudaError_t dir_set_attributes();
// bytes[t] = direction bytes of task t (bucket position), bytes[n] = 0;
// *nchk += the checked 16-bit regions among them
void dir_sizes(bool xdrop, const KParams &kp, uint64_t *bytes, unsigned long long *nchk, int grid,
               cudaStream_t st);
// *t1 = end of the arena chunk that starts at task t0
void dir_chunk_end(const uint64_t *doff, uint64_t t0, uint64_t n, uint64_t budget, uint64_t *t1,
                   cudaStream_t st);
// DP of the tasks [t0, t1) (grid blocks, dyn bytes of dynamic shared memory),
// with kp.dir16_pair (X-drop) a pass over their half-warp regions (SW runs
// them in its common pass), with chk a pass over
// their checked 16-bit regions (each of these with its work counter
// kp.counter[0] reset first), then their traceback (grid_tb blocks of 256
// threads); returns the kernels launched
int dir_run(bool xdrop, int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
            uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st);

// the same per mode, in their own translation units (pg_dir_ga.cu, pg_dir_sw.cu)
cudaError_t dir_set_attributes_ga();
cudaError_t dir_set_attributes_sw();
int dir_run_ga(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
               uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st);
int dir_run_sw(int tie, const KParams &kp, uint64_t t0, uint64_t t1, const uint64_t *doff,
               uint8_t *arena, int *dsc, int grid, int dyn, int grid_tb, bool chk, cudaStream_t st);

}  // namespace pg
