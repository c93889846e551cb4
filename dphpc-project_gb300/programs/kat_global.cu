// Per-rank privatisation of globals and function statics, written the way
// the source converter rewrites them (source_converter/converter.cpp:130-177:
// `__device__ T name[MAX_RANKS]` with the initializer replicated per rank and
// every use wrapped in __gpu_global).  Checks follow the reference's
// toolchain_tests/global_var/global_var.c:35-60.  Compiled for at most 16
// ranks (GPU_MPI_MAX_RANKS=16).  Prints "global_var rank <r> ok <0|1>".
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stddef.h.cuh"

__device__ int g1[16] = {-15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15, -15};
__device__ int g2[16][2] = {{ -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }, { -1, -2 }};
__device__ int* g3[16][3] = {{NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}, {NULL, NULL, NULL}};
__device__ int g4[16][2][3] = {{{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}, {{1,2,3},{4,5,6}}};
__device__ int foo_x[16][10] = {{4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}, {4,5,6,7}};
__device__ int main_g5[16][10] = {{1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}, {1,2}};

#define MACRO_g2 __gpu_global(g2)

__device__ int foo() {
    __gpu_global(foo_x)[3] += 1;
    return __gpu_global(foo_x)[3];
}

__device__ int __gpu_main(int argc, char** argv) {
    MPI_Init(0, 0);
    int rank = -1;
    int error = 0;
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    if (__gpu_global(g1) != -15) error = 1;
    if (__gpu_global(g2)[0] != -1) error = 1;
    if (__gpu_global(g2)[1] != -2) error = 1;
    __gpu_global(g1) = rank;
    MACRO_g2[0] = rank + 1;
    MACRO_g2[1] = rank + 2;
    __gpu_global(g3)[2] = ((int*)NULL) + rank + 3;
    __gpu_global(g4)[1][1] = rank + 4;
    foo();
    foo();
    MPI_Barrier(MPI_COMM_WORLD);
    int foo_res = foo();
    if (__gpu_global(g1) != rank) error = 1;
    if (__gpu_global(g2)[0] != rank + 1) error = 1;
    if (__gpu_global(g2)[1] != rank + 2) error = 1;
    if (__gpu_global(g3)[2] != ((int*)NULL) + rank + 3) error = 1;
    if (__gpu_global(g4)[1][1] != rank + 4) error = 1;
    if (__gpu_global(g4)[1][2] != 6) error = 1;
    if (__gpu_global(main_g5)[1] != 2) error = 1;
    if (foo_res != 10) error = 1;
    printf("global_var rank %d ok %d\n", rank, !error);
    MPI_Finalize();
    return error;
}

__device__ int __gpu_max_threads() { return 16; }
