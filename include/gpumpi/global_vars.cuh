#pragma once

// Per-rank privatisation of converted globals.
//
// The converter turns every global `T x` into `__device__ T x[MAX_RANKS]` and
// every use into `__gpu_global(x)` (source_converter/converter.cpp:130-177).
// The reference indexes by global thread id (gpu_main/global_vars.cuh:15);
// here a rank is a thread block, and the index is the rank's slot: unique
// among all ranks of all jobs that run at the same time, also when several
// jobs run as separate kernels side by side.  The runtime keeps the slot in
// the first int of the block's dynamic shared memory, and the launcher refuses
// slots beyond __gpu_max_threads().
extern __shared__ __align__(16) char __gpumpi_dsmem[];
#define __gpu_global(var) (var[*(const int*)__gpumpi_dsmem])

#ifndef GPU_MPI_MAX_RANKS
#define GPU_MPI_MAX_RANKS 1024
#endif
