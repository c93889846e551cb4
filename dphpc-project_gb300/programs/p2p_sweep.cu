// Point-to-point sweep as an MPI program (converter-output form).
//
// Pattern "pairs": rank r exchanges with r^1 (an odd last rank idles);
// pattern "ring": rank r sends to r+1 and receives from r-1 (mod P).
// Mode "block": MPI_Send/MPI_Recv, ordered by rank parity so that no rank
// waits on a send that nobody receives; mode "nb": MPI_Irecv + MPI_Isend +
// MPI_Waitall.  For every size b = 2^lg bytes, lg in [lg_min, lg_max], each
// rank allocates its buffers with malloc, fills the send buffer with a
// splitmix64 stream seeded by (rank, lg), and runs `iters` exchanges; the
// first 8 bytes of every message carry (sender, iteration) and are checked on
// every receive, the whole payload after the last one.  Rank 0 prints, per
// size, the error count and a checksum of every received byte (equal between
// a GPU run and a host MPI run), then on a separate line the time of the
// slowest rank and the algorithmic bandwidth (2b per message).  With "dup"
// the exchanges run on a duplicate of MPI_COMM_WORLD (same ranks, its own
// context) instead of MPI_COMM_WORLD itself.
// Usage: p2p_sweep pairs|ring block|nb lg_min lg_max iters [world|dup] ---gpumpi -n P
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"

__device__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ unsigned long long word_of(int rank, int lg, long i) {
    return mix64(((unsigned long long)rank << 40) ^ ((unsigned long long)lg << 32) ^ (unsigned long long)i);
}

__device__ unsigned long long stamp_of(int rank, int it) {
    return 0x5A00000000000000ull | ((unsigned long long)rank << 24) | (unsigned long long)it;
}

__device__ int exchange(int pattern, int mode, int rank, int size, void* sbuf, void* rbuf, long b,
                        int* src_out, MPI_Comm comm) {
    int dst, src;
    if (pattern == 0) {
        dst = rank ^ 1;
        src = dst;
        if (dst >= size) {
            *src_out = -1;
            return 0;
        }
    } else {
        dst = (rank + 1) % size;
        src = (rank + size - 1) % size;
    }
    *src_out = src;
    int rc = 0;
    if (mode == 0) {
        if ((rank & 1) == 0) {
            rc |= MPI_Send(sbuf, (int)b, MPI_BYTE, dst, 7, comm);
            rc |= MPI_Recv(rbuf, (int)b, MPI_BYTE, src, 7, comm, MPI_STATUS_IGNORE);
        } else {
            rc |= MPI_Recv(rbuf, (int)b, MPI_BYTE, src, 7, comm, MPI_STATUS_IGNORE);
            rc |= MPI_Send(sbuf, (int)b, MPI_BYTE, dst, 7, comm);
        }
    } else {
        MPI_Request req[2];
        rc |= MPI_Irecv(rbuf, (int)b, MPI_BYTE, src, 7, comm, &req[0]);
        rc |= MPI_Isend(sbuf, (int)b, MPI_BYTE, dst, 7, comm, &req[1]);
        rc |= MPI_Waitall(2, req, MPI_STATUSES_IGNORE);
    }
    return rc;
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    if (argc < 6 || size < 2) {
        if (rank == 0) printf("usage: p2p_sweep pairs|ring block|nb lg_min lg_max iters [world|dup] (2+ ranks)\n");
        MPI_Finalize();
        return 1;
    }
    const int pattern = strcmp(argv[1], "ring") == 0 ? 1 : 0;
    const int mode = strcmp(argv[2], "nb") == 0 ? 1 : 0;
    const int lg_min = atoi(argv[3]) < 3 ? 3 : atoi(argv[3]);
    const int lg_max = atoi(argv[4]);
    const int iters = atoi(argv[5]) < 1 ? 1 : atoi(argv[5]);
    MPI_Comm comm = MPI_COMM_WORLD;
    if (argc > 6 && strcmp(argv[6], "dup") == 0) MPI_Comm_dup(MPI_COMM_WORLD, &comm);
    int status = 0;
    for (int lg = lg_min; lg <= lg_max; lg++) {
        const long b = 1L << lg;
        const long nw = b / 8;
        unsigned long long* sbuf = (unsigned long long*)malloc(b);
        unsigned long long* rbuf = (unsigned long long*)malloc(b);
        long errors = 0;
        // every rank must have its buffers, or no rank exchanges at this size
        int ok = sbuf && rbuf, all_ok = 0;
        MPI_Allreduce(&ok, &all_ok, 1, MPI_INT, MPI_MIN, MPI_COMM_WORLD);
        if (!all_ok) {
            if (rank == 0) printf("p2p bytes %ld: out of device heap (raise -p)\n", b);
            free(sbuf);
            free(rbuf);
            status = 1;
            break;
        }
        for (long i = 0; i < nw; i++) sbuf[i] = word_of(rank, lg, i);
        memset(rbuf, 0, b);
        MPI_Barrier(MPI_COMM_WORLD);
        double t0 = MPI_Wtime();
        int src = -1;
        for (int it = 0; it < iters; it++) {
            sbuf[0] = stamp_of(rank, it);
            if (exchange(pattern, mode, rank, size, sbuf, rbuf, b, &src, comm) != MPI_SUCCESS) errors++;
            if (src >= 0 && rbuf[0] != stamp_of(src, it)) errors++;
        }
        double t1 = MPI_Wtime();
        unsigned long long check = 0;
        if (src >= 0) {
            for (long i = 1; i < nw; i++) {
                if (rbuf[i] != word_of(src, lg, i)) errors++;
                check += mix64(rbuf[i] ^ (unsigned long long)i);
            }
            check += mix64(rbuf[0]);
        }
        double dt = t1 - t0, tmax = 0.0;
        long errs_total = 0;
        unsigned long long check_total = 0;
        MPI_Reduce(&dt, &tmax, 1, MPI_DOUBLE, MPI_MAX, 0, MPI_COMM_WORLD);
        MPI_Reduce(&errors, &errs_total, 1, MPI_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
        MPI_Reduce(&check, &check_total, 1, MPI_UNSIGNED_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
        if (rank == 0) {
            const long msgs = pattern == 0 ? (long)(size / 2) * 2 : (long)size;
            const double bytes = 2.0 * (double)b * (double)msgs * (double)iters;
            printf("p2p %s %s ranks %d bytes %ld iters %d errors %ld checksum %016llx\n", pattern ? "ring" : "pairs",
                   mode ? "nb" : "block", size, b, iters, errs_total, check_total);
            printf("p2p-time bytes %ld seconds %.6f us_per_iter %.3f GBps %.3f\n", b, tmax, 1e6 * tmax / iters,
                   tmax > 0 ? bytes / tmax / 1e9 : 0.0);
            if (errs_total) status = 1;
        }
        free(sbuf);
        free(rbuf);
    }
    if (comm != MPI_COMM_WORLD) MPI_Comm_free(&comm);
    MPI_Finalize();
    return status;
}

__device__ int __gpu_max_threads() { return 1024; }
