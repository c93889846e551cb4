// Allocator known answers (converter-output form), after the reference's
// allocator tests (gpu_libs/gpu_malloc/dynamic_allocator/tests.cu:12-120 and
// alignment_tests.cu): sizes from 1 byte to several MiB come back non-NULL,
// 16-byte aligned and disjoint (every object keeps its own pattern while all
// are live); freed space is reused (alternate frees and reallocations, and a
// growing sequence of large blocks that only fits if freed runs merge);
// calloc returns zeros; realloc keeps the prefix; free(NULL) is harmless.
// Each rank prints "kat_malloc rank r ok" or the first failure.
// Usage: kat_malloc [rounds=4] ---gpumpi -n P   (run with -p of at least 256M per rank set)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"

#define NSIZES 24

__device__ unsigned char pat(int rank, int k, long i) { return (unsigned char)(rank * 131 + k * 31 + i * 7 + 1); }

__device__ int fill_check(unsigned char* p, long n, int rank, int k, int check) {
    // whole object for small sizes; first/last 4 KiB and a stride for large ones
    for (long i = 0; i < n; i++) {
        if (n > 65536 && i >= 4096 && i < n - 4096 && (i % 4093) != 0) continue;
        if (check) {
            if (p[i] != pat(rank, k, i)) return 0;
        } else {
            p[i] = pat(rank, k, i);
        }
    }
    return 1;
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    const int rounds = argc > 1 ? atoi(argv[1]) : 4;
    const long sizes[NSIZES] = {1,     2,     3,      8,       15,      16,      17,          31,
                                64,    100,   1000,   4095,    4096,    4097,    32768,       32769,
                                65535, 65536, 100000, 1 << 20, 3 << 20, 655361, (1 << 22) + 5, 12345};
    unsigned char* obj[NSIZES];
    const char* fail = nullptr;
    for (int r = 0; r < rounds && !fail; r++) {
        for (int k = 0; k < NSIZES && !fail; k++) {
            obj[k] = (unsigned char*)malloc(sizes[k]);
            if (!obj[k]) fail = "malloc returned NULL";
            else if (((unsigned long long)obj[k] & 15) != 0) fail = "pointer not 16-byte aligned";
            else fill_check(obj[k], sizes[k], rank, k + r, 0);
        }
        for (int k = 0; k < NSIZES && !fail; k++)
            if (!fill_check(obj[k], sizes[k], rank, k + r, 1)) fail = "objects overlap";
        // free every other object, allocate the same sizes again, check everything
        for (int k = 0; k < NSIZES && !fail; k += 2) {
            free(obj[k]);
            obj[k] = (unsigned char*)malloc(sizes[k]);
            if (!obj[k]) fail = "malloc after free returned NULL";
            else fill_check(obj[k], sizes[k], rank, k + r + 100, 0);
        }
        for (int k = 0; k < NSIZES && !fail; k++)
            if (!fill_check(obj[k], sizes[k], rank, k % 2 == 0 ? k + r + 100 : k + r, 1)) fail = "reuse overlaps";
        for (int k = 0; k < NSIZES; k++)
            if (!fail) free(obj[k]);
    }
    // growing large blocks: each size is freed before the next, larger one; without
    // merging of freed runs the sequence needs the sum of all sizes
    for (int lg = 16; lg <= 24 && !fail; lg++) {
        unsigned char* a = (unsigned char*)malloc(1L << lg);
        unsigned char* b = (unsigned char*)malloc(1L << lg);
        if (!a || !b) fail = "growing large blocks: NULL";
        else {
            fill_check(a, 1L << lg, rank, lg, 0);
            fill_check(b, 1L << lg, rank, lg + 50, 0);
            if (!fill_check(a, 1L << lg, rank, lg, 1) || !fill_check(b, 1L << lg, rank, lg + 50, 1))
                fail = "growing large blocks overlap";
        }
        free(a);
        free(b);
    }
    if (!fail) {
        int* z = (int*)calloc(5000, sizeof(int));
        if (!z) fail = "calloc returned NULL";
        else {
            for (int i = 0; i < 5000; i++)
                if (z[i] != 0) fail = "calloc memory not zero";
            for (int i = 0; i < 5000; i++) z[i] = i * rank;
            int* y = (int*)realloc(z, 200000 * sizeof(int));
            if (!y) fail = "realloc returned NULL";
            else {
                for (int i = 0; i < 5000; i++)
                    if (y[i] != i * rank) fail = "realloc lost the prefix";
                free(y);
            }
        }
        free(nullptr);
    }
    if (fail) printf("kat_malloc rank %d FAILED: %s\n", rank, fail);
    else printf("kat_malloc rank %d ok\n", rank);
    MPI_Finalize();
    return fail ? 1 : 0;
}

__device__ int __gpu_max_threads() { return 1024; }
