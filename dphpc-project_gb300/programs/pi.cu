// pi by the midpoint rule on 4/(1+x^2) over [0,1], in the form the source
// converter emits (main -> __gpu_main, __device__ functions, .cuh includes).
// Decomposition as in toolchain_tests/pi/cpi.c:45-56: rank r sums intervals
// r+1, r+1+P, ... in order, then MPI_Reduce(SUM, DOUBLE) to rank 0.
// Usage: pi [N] ---gpumpi -n P      (default N = 10^7)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "math.h.cuh"

__device__ double f(double a) { return 4.0 / (1.0 + a * a); }

__device__ int __gpu_main(int argc, char** argv) {
    int n = 10000000, myid, numprocs, i;
    double PI25DT = 3.141592653589793238462643;
    double mypi, pi, h, sum, x;
    double startwtime = 0.0, endwtime;

    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &numprocs);
    MPI_Comm_rank(MPI_COMM_WORLD, &myid);
    if (myid == 0) {
        if (argc > 1) n = atoi(argv[1]);
        startwtime = MPI_Wtime();
    }
    MPI_Bcast(&n, 1, MPI_INT, 0, MPI_COMM_WORLD);

    h = 1.0 / (double)n;
    sum = 0.0;
    for (i = myid + 1; i <= n; i += numprocs) {
        x = h * ((double)i - 0.5);
        sum += f(x);
    }
    mypi = h * sum;

    MPI_Reduce(&mypi, &pi, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);

    if (myid == 0) {
        unsigned long long bits;
        endwtime = MPI_Wtime();
        memcpy(&bits, &pi, sizeof(bits));
        printf("pi is approximately %.16f, Error is %.16f\n", pi, fabs(pi - PI25DT));
        printf("pi bits %016llx n %d ranks %d\n", bits, n, numprocs);
        printf("wall clock time = %f\n", endwtime - startwtime);
    }
    MPI_Finalize();
    return 0;
}

__device__ int __gpu_max_threads() { return 1024; }
