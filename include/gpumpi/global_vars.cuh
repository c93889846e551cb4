#pragma once

// Per-rank privatisation of converted globals.
//
// The converter turns every global `T x` into `__device__ T x[MAX_RANKS]` and
// every use into `__gpu_global(x)` (source_converter/converter.cpp:130-177).
// The reference indexes by global thread id (gpu_main/global_vars.cuh:15);
// here a rank is a thread block, so the index is the block's slot in the
// launch.  Slots are unique among all ranks of all jobs that run at the same
// time, and the launcher refuses grids larger than __gpu_max_threads().
#define __gpu_global(var) (var[blockIdx.x])

#ifndef GPU_MPI_MAX_RANKS
#define GPU_MPI_MAX_RANKS 1024
#endif
