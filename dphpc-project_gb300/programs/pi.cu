// Midpoint-rule estimate of pi = integral of 4/(1+x^2) over [0,1], as an MPI
// program in converter-output form (__gpu_main, __device__ functions, .cuh
// includes).  Interval k (1-based) has midpoint h*(k - 1/2); rank r takes the
// intervals r+1, r+1+P, r+1+2P, ... (the decomposition of the reference's pi
// test, toolchain_tests/pi/cpi.c:45-56), the rank sums are reduced to rank 0
// with MPI_Reduce(MPI_SUM, MPI_DOUBLE) in rank order, and rank 0 prints the
// estimate in the reference program's result-line format.
//
// Local sum: by default one running sum over the rank's intervals in order
// (the reference program's order, so the result line equals its output
// bit for bit).  With a chunk count K > 0 the rank's intervals are cut into
// K consecutive runs summed by a parallel loop (every iteration one run, in
// order) and the K run sums are added in run order: the same arithmetic on
// the GPU and in a host build, so the two still agree bit for bit.
// Usage: pi [N [K]] ---gpumpi -n P      (default N = 10^7, K = 0)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "math.h.cuh"
#include "omp.h.cuh"

__device__ double integrand(double x) { return 4.0 / (1.0 + x * x); }

struct runs {
    long first;      // the rank's first interval (1-based)
    long stride;     // ranks
    long count;      // the rank's intervals
    long nruns;
    double width;    // interval width h
    double* part;    // [nruns] run sums
};

__device__ void sum_run(long k, void* arg) {
    struct runs* r = (struct runs*)arg;
    const long lo = k * r->count / r->nruns, hi = (k + 1) * r->count / r->nruns;
    double acc = 0.0;
    for (long j = lo; j < hi; j++) {
        const long iv = r->first + j * r->stride;
        acc += integrand(r->width * ((double)iv - 0.5));
    }
    r->part[k] = acc;
}

__device__ int __gpu_main(int argc, char** argv) {
    int nint = 10000000, nruns = 0, rank = 0, size = 1;
    double t_start = 0.0;
    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    if (rank == 0) {
        if (argc > 1) nint = atoi(argv[1]);
        if (argc > 2) nruns = atoi(argv[2]);
        t_start = MPI_Wtime();
    }
    int params[2] = {nint, nruns};
    MPI_Bcast(params, 2, MPI_INT, 0, MPI_COMM_WORLD);
    nint = params[0];
    nruns = params[1];

    const double width = 1.0 / (double)nint;
    double local = 0.0;
    if (nruns <= 0) {
        for (int iv = rank + 1; iv <= nint; iv += size) local += integrand(width * ((double)iv - 0.5));
    } else {
        struct runs* r = (struct runs*)malloc(sizeof(struct runs));
        r->first = rank + 1;
        r->stride = size;
        r->count = rank + 1 <= nint ? (nint - (rank + 1)) / size + 1 : 0;
        r->nruns = nruns;
        r->width = width;
        r->part = (double*)malloc(sizeof(double) * nruns);
        gpumpi_parallel_for(nruns, sum_run, r);
        for (int k = 0; k < nruns; k++) local += r->part[k];
        free(r->part);
        free(r);
    }
    double mine = width * local, total = 0.0;
    MPI_Reduce(&mine, &total, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);

    if (rank == 0) {
        const double elapsed = MPI_Wtime() - t_start;
        const double ref = 3.141592653589793238462643;
        unsigned long long bits;
        memcpy(&bits, &total, sizeof(bits));
        printf("pi is approximately %.16f, Error is %.16f\n", total, fabs(total - ref));
        printf("pi bits %016llx n %d ranks %d\n", bits, nint, size);
        printf("wall clock time = %f\n", elapsed);
    }
    MPI_Finalize();
    return 0;
}

__device__ int __gpu_max_threads() { return 1024; }
