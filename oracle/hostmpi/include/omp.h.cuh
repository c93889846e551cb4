#pragma once
#include "global_vars.cuh"
static inline int omp_get_max_threads(void) { return 1; }
static inline int omp_get_num_threads(void) { return 1; }
static inline int omp_get_thread_num(void) { return 0; }
// The rank-block parallel loop of the GPU runtime, run in order on the host.
static inline void gpumpi_parallel_for(long n, void (*body)(long, void*), void* arg) {
    for (long i = 0; i < n; i++) body(i, arg);
}
// The block of the rank running a loop iteration: a host rank is one block.
static inline int gpumpi_loop_block(void) { return 0; }
static inline void gpumpi_atomic_add_i64(long long* p, long long v) {
    *p = (long long)((unsigned long long)*p + (unsigned long long)v);
}
static inline int gpumpi_atomic_add_i32(int* p, int v) {
    int old = *p;
    *p = (int)((unsigned)old + (unsigned)v);
    return old;
}
