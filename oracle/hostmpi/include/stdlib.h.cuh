#pragma once
#include "global_vars.cuh"
#include <stdlib.h>
#include <stddef.h>
#ifdef __cplusplus
static inline void* hostmpi_malloc_any(size_t n, bool coalesced = false) { (void)coalesced; return malloc(n); }
static inline void* hostmpi_calloc_any(size_t n, size_t s, bool coalesced = false) { (void)coalesced; return calloc(n, s); }
#define malloc(...) hostmpi_malloc_any(__VA_ARGS__)
#define calloc(...) hostmpi_calloc_any(__VA_ARGS__)
#endif
static inline void __gpu_init_malloc(void) {}
static inline void __gpu_clean_malloc(void) {}
