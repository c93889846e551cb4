#pragma once
#include "gpumpi_prelude.cuh"
#define omp_get_max_threads __gpu_omp_get_max_threads
#define omp_get_num_threads __gpu_omp_get_num_threads
#define omp_get_thread_num __gpu_omp_get_thread_num
#define omp_get_wtime __gpu_omp_get_wtime
#define gpumpi_parallel_for __gpu_parallel_for
#define gpumpi_loop_block __gpu_loop_block
// 64-bit integer add that concurrent loop iterations may apply to the same
// word (exact, so its result does not depend on their order).
__device__ inline void gpumpi_atomic_add_i64(long long* p, long long v) {
    atomicAdd((unsigned long long*)p, (unsigned long long)v);
}
// 32-bit form; returns the value before the add.
__device__ inline int gpumpi_atomic_add_i32(int* p, int v) { return atomicAdd(p, v); }
