#pragma once
// <stdlib.h> for converted programs (names as in gpu_libs/gpu_libc/stdlib.h.cuh).
// Every allocator version the converter can select maps to the same slab
// allocator; the extra `coalesced` argument those versions take is accepted
// and ignored.
#include "gpumpi_prelude.cuh"
#undef RAND_MAX
#define RAND_MAX __gpu_RAND_MAX
#define qsort __gpu_qsort
#define bsearch __gpu_bsearch
#define atoi __gpu_atoi
#define atol __gpu_atol
#define atoll __gpu_atoll
#define atof __gpu_atof
#define strtol __gpu_strtol
#define strtoul __gpu_strtoul
#define strtoll __gpu_strtoll
#define strtoull __gpu_strtoull
#define strtod __gpu_strtod
#define strtof __gpu_strtof
#define realloc __gpu_realloc
#define srand __gpu_srand
#define rand __gpu_rand
#define getenv __gpu_getenv
#define exit __gpu_exit
#define abort __gpu_abort
#define posix_memalign __gpu_posix_memalign
#define aligned_alloc __gpu_aligned_alloc
#define malloc(...) __gpu_malloc_any(__VA_ARGS__)
#define calloc(...) __gpu_calloc_any(__VA_ARGS__)
#define free __gpu_free
__device__ inline void* __gpu_malloc_any(size_t size, bool coalesced = false) {
    (void)coalesced;
    return __gpu_malloc(size);
}
__device__ inline void* __gpu_calloc_any(size_t n, size_t size, bool coalesced = false) {
    (void)coalesced;
    return __gpu_calloc(n, size);
}
#define __gpu_init_malloc_v6 __gpu_init_malloc
#define __gpu_clean_malloc_v6 __gpu_clean_malloc
