// Batched collectives as an MPI program (converter-output form): the ranks are
// split into communicators of uneven sizes (4..256, 1024 ranks in total for a
// full run; smaller worlds use a prefix of the size list and give the rest to
// the last communicator); each communicator runs Bcast, Allreduce(SUM) and
// Alltoall on int32 data uniform in [-2^20, 2^20) and FP64 data uniform in
// [-1, 1), count elements per rank (Alltoall: count / P elements per peer).
// Data come from a seeded splitmix64 hash of (rank, element, iteration).
// Rank 0 prints a checksum of every result (bit pattern based, so GPU and
// host runs must agree bit for bit) and the algorithmic bandwidth.
// Usage: coll_bench [log2(count)] [iterations] ---gpumpi -n <ranks>
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "stdint.h.cuh"

__device__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ int comm_color(int rank, int world, int* csize) {
    const int sizes[16] = {4, 8, 12, 16, 24, 32, 40, 48, 56, 64, 72, 80, 88, 96, 128, 256};
    int start = 0;
    for (int c = 0; c < 16; c++) {
        int s = sizes[c];
        if (c == 15 || start + s > world) s = world - start;
        if (rank < start + s) {
            *csize = s;
            return c;
        }
        start += s;
    }
    *csize = 1;
    return 15;
}

__device__ unsigned long long fold_sum(const void* buf, long n, int esize) {
    unsigned long long h = 0;
    const unsigned char* p = (const unsigned char*)buf;
    for (long i = 0; i < n; i++) {
        unsigned long long v = 0;
        for (int b = 0; b < esize; b++) v |= (unsigned long long)p[i * esize + b] << (8 * b);
        h += mix64(v ^ (unsigned long long)i);
    }
    return h;
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, world;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &world);
    int lg = argc > 1 ? atoi(argv[1]) : 10;
    int iters = argc > 2 ? atoi(argv[2]) : 1;
    long n = 1L << lg;
    int csize = 0;
    int color = comm_color(rank, world, &csize);
    MPI_Comm comm;
    MPI_Comm_split(MPI_COMM_WORLD, color, rank, &comm);
    int cr, P;
    MPI_Comm_rank(comm, &cr);
    MPI_Comm_size(comm, &P);
    long per = n / P;

    int* bi = (int*)malloc(sizeof(int) * n);
    double* bd = (double*)malloc(sizeof(double) * n);
    int* si = (int*)malloc(sizeof(int) * n);
    int* ri = (int*)malloc(sizeof(int) * n);
    double* sd = (double*)malloc(sizeof(double) * n);
    double* rd = (double*)malloc(sizeof(double) * n);
    int* ai = (int*)malloc(sizeof(int) * per * P + 4);
    int* bi2 = (int*)malloc(sizeof(int) * per * P + 4);
    double* ad = (double*)malloc(sizeof(double) * per * P + 8);
    double* bd2 = (double*)malloc(sizeof(double) * per * P + 8);
    if (!bi || !bd || !si || !ri || !sd || !rd || !ai || !bi2 || !ad || !bd2) {
        printf("rank %d: allocation failed\n", rank);
        MPI_Abort(MPI_COMM_WORLD, 2);
    }
    unsigned long long check = 0;
    double t_total = 0.0;
    for (int it = 0; it < iters; it++) {
        for (long i = 0; i < n; i++) {
            unsigned long long h1 = mix64(((unsigned long long)rank << 40) ^ ((unsigned long long)it << 34) ^ (unsigned long long)i);
            unsigned long long h2 = mix64(h1);
            si[i] = (int)(h1 % 2097152ull) - 1048576;
            sd[i] = (double)(h2 >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
            bi[i] = cr == 0 ? si[i] : 0;
            bd[i] = cr == 0 ? sd[i] : 0.0;
        }
        for (long i = 0; i < per * P; i++) {
            ai[i] = si[i];
            ad[i] = sd[i];
        }
        MPI_Barrier(MPI_COMM_WORLD);
        double t0 = MPI_Wtime();
        MPI_Bcast(bi, (int)n, MPI_INT, 0, comm);
        MPI_Bcast(bd, (int)n, MPI_DOUBLE, 0, comm);
        MPI_Allreduce(si, ri, (int)n, MPI_INT, MPI_SUM, comm);
        MPI_Allreduce(sd, rd, (int)n, MPI_DOUBLE, MPI_SUM, comm);
        MPI_Alltoall(ai, (int)per, MPI_INT, bi2, (int)per, MPI_INT, comm);
        MPI_Alltoall(ad, (int)per, MPI_DOUBLE, bd2, (int)per, MPI_DOUBLE, comm);
        MPI_Barrier(MPI_COMM_WORLD);
        t_total += MPI_Wtime() - t0;
        check += fold_sum(bi, n, 4) + 3 * fold_sum(bd, n, 8) + 5 * fold_sum(ri, n, 4) +
                 7 * fold_sum(rd, n, 8) + 11 * fold_sum(bi2, per * P, 4) + 13 * fold_sum(bd2, per * P, 8);
    }
    unsigned long long all = 0;
    MPI_Reduce(&check, &all, 1, MPI_UNSIGNED_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    // algorithmic bytes of one iteration, summed over communicators (each
    // communicator's rank 0 contributes its communicator's share)
    double bytes = 0.0;
    if (cr == 0) {
        double b4 = 4.0 * n, b8 = 8.0 * n;
        bytes = P * (b4 + b8) + 2.0 * P * (b4 + b8) + 2.0 * P * P * per * 12.0;
    }
    double total_bytes = 0.0, tmax = 0.0;
    MPI_Reduce(&bytes, &total_bytes, 1, MPI_DOUBLE, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce(&t_total, &tmax, 1, MPI_DOUBLE, MPI_MAX, 0, MPI_COMM_WORLD);
    if (rank == 0) {
        printf("coll_bench checksum %016llx ranks %d count %ld iters %d\n", all, world, n, iters);
        printf("coll_bench time %.6f s bytes %.0f GBps %.3f\n", tmax, total_bytes * iters,
               tmax > 0 ? total_bytes * iters / tmax / 1e9 : 0.0);
    }
    free(bi);
    free(bd);
    free(si);
    free(ri);
    free(sd);
    free(rd);
    free(ai);
    free(bi2);
    free(ad);
    free(bd2);
    MPI_Comm_free(&comm);
    MPI_Finalize();
    return 0;
}

__device__ int __gpu_max_threads() { return 1024; }
