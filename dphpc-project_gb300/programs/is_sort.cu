// Integer bucket sort in the style of the NAS IS kernel, as an MPI program
// (converter-output form).  Written from the algorithm's description; no NPB
// source, key generator or verification table is used.
//
// Keys: total_keys int32 values spread evenly over the ranks,
// key = floor(2^max_lg * (u1+u2+u3+u4)/4) with u uniform in [0,1) from a
// splitmix64 stream seeded by (rank, index).  Buckets: 2^nb_lg by the key's top
// bits.  Each of `iters` iterations (numbered 1..iters):
//   1. rank 0 overwrites two keys: key[it] = it, key[it+iters] = max_key - it
//      (the per-iteration perturbation of IS, is.c:647-650)
//   2. local bucket histogram, MPI_Allreduce(SUM) of the histograms
//   3. buckets are assigned to ranks in order, each rank taking buckets until
//      its cumulative share of the total reaches (r+1)/P
//   4. MPI_Alltoall of the per-destination key counts
//   5. local bucket sort into the send buffer, MPI_Alltoallv of the keys
//   6. counting sort of the received keys over the rank's key range
// Rank 0 prints one checksum line per iteration (received counts and a hash
// of each rank's key-rank array, reduced in rank order), then after the last
// iteration the full verification: every rank's keys nondecreasing and each
// rank's first key >= the previous rank's last key.
//
// The key loops run through gpumpi_parallel_for (omp.h.cuh): on the GPU over
// the rank's whole thread block, in a host build in order.  The keys are cut
// into NCHUNK fixed chunks; each chunk counts its own bucket histogram, and
// the chunks' counts give every chunk its write offsets, so the bucket sort
// places keys exactly where a serial loop would.  The counting sort counts
// with exact integer atomic adds, whose result does not depend on order.
// Usage: is_sort [log2(total keys)=23] [iters=10] [log2(max key)=19] [log2(buckets)=10]
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "omp.h.cuh"

#define NCHUNK 256

__device__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Four uniforms in [0, 2^16) from one 64-bit hash; their sum scaled to the key range.
__device__ int make_key(int rank, long i, int max_lg) {
    unsigned long long h = mix64(((unsigned long long)rank << 44) ^ (unsigned long long)i);
    unsigned long long s = (h & 0xffff) + ((h >> 16) & 0xffff) + ((h >> 32) & 0xffff) + (h >> 48);
    // (u1+u2+u3+u4)/4 with u = v / 2^16, times 2^max_lg
    return (int)((s << max_lg) >> 18);
}

// State shared by the loop bodies (in the heap).
struct Is {
    int rank, max_lg, nbuckets, shift, lo_key, range;
    long nkeys, nrecv;
    int* keys;
    int* sendk;
    int* recvk;
    int* sorted;
    int* chist;    // [NCHUNK][nbuckets] per-chunk bucket counts, then write offsets
    int* hist;     // [nbuckets] this rank's bucket counts
    int* bstart;   // [nbuckets] first position of each bucket in the send buffer
    int* cnt;      // [range + 1] counting-sort counts, then key ranks
    long* bad;     // [NCHUNK] received keys outside the range, per chunk
    int* csum;     // [NCHUNK] per-chunk sums of cnt, then their exclusive prefix
};

__device__ void chunk_range(long n, int c, long* k0, long* k1) {
    *k0 = n * c / NCHUNK;
    *k1 = n * (c + 1) / NCHUNK;
}

__device__ void gen_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    long k0, k1;
    chunk_range(s->nkeys, (int)c, &k0, &k1);
    for (long i = k0; i < k1; i++) s->keys[i] = make_key(s->rank, i, s->max_lg);
}

__device__ void hist_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    int* h = s->chist + c * s->nbuckets;
    for (int b = 0; b < s->nbuckets; b++) h[b] = 0;
    long k0, k1;
    chunk_range(s->nkeys, (int)c, &k0, &k1);
    for (long i = k0; i < k1; i++) h[s->keys[i] >> s->shift]++;
}

__device__ void bucket_total(long b, void* arg) {
    Is* s = (Is*)arg;
    const int* h = s->chist + b;
    const int nb = s->nbuckets;
    int t = 0;
    for (int c = 0; c < NCHUNK; c += 8) {
        int v[8];
        for (int k = 0; k < 8; k++) v[k] = h[(c + k) * nb];
        for (int k = 0; k < 8; k++) t += v[k];
    }
    s->hist[b] = t;
}

// Bucket b: each chunk's counts turned into its write offsets.
__device__ void bucket_offsets(long b, void* arg) {
    Is* s = (Is*)arg;
    int* h = s->chist + b;
    const int nb = s->nbuckets;
    int run = s->bstart[b];
    // 8 counts read before any is overwritten: the reads do not wait on the writes
    for (int c = 0; c < NCHUNK; c += 8) {
        int v[8];
        for (int k = 0; k < 8; k++) v[k] = h[(c + k) * nb];
        for (int k = 0; k < 8; k++) {
            h[(c + k) * nb] = run;
            run += v[k];
        }
    }
}

__device__ void scatter_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    int* off = s->chist + c * s->nbuckets;
    long k0, k1;
    chunk_range(s->nkeys, (int)c, &k0, &k1);
    for (long i = k0; i < k1; i++) {
        const int key = s->keys[i];
        s->sendk[off[key >> s->shift]++] = key;
    }
}

__device__ void clear_counts(long k, void* arg) { ((Is*)arg)->cnt[k] = 0; }

// Inclusive prefix sum of cnt[0..range] in three passes (chunk sums, their
// exclusive scan, then each chunk's running sum): the same integers as the
// serial loop, computed by the whole rank block.
__device__ void prefix_sum_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    long k0, k1;
    chunk_range(s->range + 1, (int)c, &k0, &k1);
    const int* cnt = s->cnt;
    int t = 0;
    for (long k = k0; k < k1; k++) t += cnt[k];
    s->csum[c] = t;
}

__device__ void prefix_apply_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    long k0, k1;
    chunk_range(s->range + 1, (int)c, &k0, &k1);
    int* cnt = s->cnt;
    int run = s->csum[c];
    for (long k = k0; k < k1; k++) {
        run += cnt[k];
        cnt[k] = run;
    }
}

__device__ void count_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    long k0, k1, bad = 0;
    chunk_range(s->nrecv, (int)c, &k0, &k1);
    for (long i = k0; i < k1; i++) {
        const int k = s->recvk[i] - s->lo_key;
        if (k < 0 || k >= s->range) bad++;
        else gpumpi_atomic_add_i32(&s->cnt[k + 1], 1);
    }
    s->bad[c] = bad;
}

// Every received key at its rank (keys of equal value are interchangeable).
__device__ void place_chunk(long c, void* arg) {
    Is* s = (Is*)arg;
    long k0, k1;
    chunk_range(s->nrecv, (int)c, &k0, &k1);
    for (long i = k0; i < k1; i++) {
        const int k = s->recvk[i] - s->lo_key;
        if (k >= 0 && k < s->range) s->sorted[gpumpi_atomic_add_i32(&s->cnt[k], 1)] = s->recvk[i];
    }
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const int total_lg = argc > 1 ? atoi(argv[1]) : 23;
    const int iters = argc > 2 ? atoi(argv[2]) : 10;
    const int max_lg = argc > 3 ? atoi(argv[3]) : 19;
    const int nb_lg = argc > 4 ? atoi(argv[4]) : 10;
    const long total = 1L << total_lg;
    const int max_key = 1 << max_lg;
    const int nbuckets = 1 << nb_lg;

    Is* s = (Is*)calloc(1, sizeof(Is));
    s->rank = rank;
    s->max_lg = max_lg;
    s->nbuckets = nbuckets;
    s->shift = max_lg - nb_lg;
    s->nkeys = total / size + (rank < total % size ? 1 : 0);
    const long nk = s->nkeys > 0 ? s->nkeys : 1;
    s->keys = (int*)malloc(sizeof(int) * nk);
    s->sendk = (int*)malloc(sizeof(int) * nk);
    s->chist = (int*)malloc(sizeof(int) * (size_t)NCHUNK * nbuckets);
    s->bstart = (int*)malloc(sizeof(int) * nbuckets);
    s->cnt = (int*)malloc(sizeof(int) * (max_key + 1));
    s->bad = (long*)malloc(sizeof(long) * NCHUNK);
    s->csum = (int*)malloc(sizeof(int) * NCHUNK);
    s->hist = (int*)malloc(sizeof(int) * nbuckets);
    int* hist = s->hist;
    int* ghist = (int*)malloc(sizeof(int) * nbuckets);
    int* owner = (int*)malloc(sizeof(int) * nbuckets);
    int* scount = (int*)malloc(sizeof(int) * size);
    int* rcount = (int*)malloc(sizeof(int) * size);
    int* sdispl = (int*)malloc(sizeof(int) * size);
    int* rdispl = (int*)malloc(sizeof(int) * size);
    long rcap = 0;
    gpumpi_parallel_for(NCHUNK, gen_chunk, s);

    MPI_Barrier(MPI_COMM_WORLD);
    const double t0 = MPI_Wtime();
    for (int it = 1; it <= iters; it++) {
        if (rank == 0 && s->nkeys > it + iters) {
            s->keys[it] = it;
            s->keys[it + iters] = max_key - it;
        }
        gpumpi_parallel_for(NCHUNK, hist_chunk, s);
        gpumpi_parallel_for(nbuckets, bucket_total, s);
        MPI_Allreduce(hist, ghist, nbuckets, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
        // bucket ownership: rank r takes buckets while its cumulative share < (r+1)/P
        long acc = 0;
        int r = 0;
        for (int b = 0; b < nbuckets; b++) {
            owner[b] = r;
            acc += ghist[b];
            while (r < size - 1 && acc * size >= (long)(r + 1) * total) r++;
        }
        for (int q = 0; q < size; q++) scount[q] = 0;
        for (int b = 0; b < nbuckets; b++) scount[owner[b]] += hist[b];
        MPI_Alltoall(scount, 1, MPI_INT, rcount, 1, MPI_INT, MPI_COMM_WORLD);
        // local bucket sort into the send buffer (buckets in order = destinations in order)
        int off = 0;
        for (int b = 0; b < nbuckets; b++) {
            s->bstart[b] = off;
            off += hist[b];
        }
        gpumpi_parallel_for(nbuckets, bucket_offsets, s);
        gpumpi_parallel_for(NCHUNK, scatter_chunk, s);
        sdispl[0] = 0;
        rdispl[0] = 0;
        for (int q = 1; q < size; q++) {
            sdispl[q] = sdispl[q - 1] + scount[q - 1];
            rdispl[q] = rdispl[q - 1] + rcount[q - 1];
        }
        s->nrecv = (long)rdispl[size - 1] + rcount[size - 1];
        if (s->nrecv > rcap) {
            free(s->recvk);
            free(s->sorted);
            rcap = s->nrecv + s->nrecv / 8 + 64;
            s->recvk = (int*)malloc(sizeof(int) * rcap);
            s->sorted = (int*)malloc(sizeof(int) * rcap);
        }
        MPI_Alltoallv(s->sendk, scount, sdispl, MPI_INT, s->recvk, rcount, rdispl, MPI_INT, MPI_COMM_WORLD);
        // key range of this rank's buckets
        int first_b = -1, last_b = -1;
        for (int b = 0; b < nbuckets; b++)
            if (owner[b] == rank) {
                if (first_b < 0) first_b = b;
                last_b = b;
            }
        s->lo_key = first_b < 0 ? 0 : first_b << s->shift;
        s->range = first_b < 0 ? 0 : ((last_b + 1) << s->shift) - s->lo_key;
        gpumpi_parallel_for(s->range + 1, clear_counts, s);
        gpumpi_parallel_for(NCHUNK, count_chunk, s);
        long bad = 0;
        for (int c = 0; c < NCHUNK; c++) bad += s->bad[c];
        // cnt[k] = rank of the first key k (inclusive prefix sum; cnt[0] = 0)
        gpumpi_parallel_for(NCHUNK, prefix_sum_chunk, s);
        {
            int run = 0;
            for (int c = 0; c < NCHUNK; c++) {
                const int t = s->csum[c];
                s->csum[c] = run;
                run += t;
            }
        }
        gpumpi_parallel_for(NCHUNK, prefix_apply_chunk, s);
        unsigned long long h = (unsigned long long)s->nrecv * 0x100000001B3ull + (unsigned long long)bad;
        for (int k = 0; k <= s->range; k += 1 + s->range / 64) h = mix64(h ^ (unsigned long long)s->cnt[k]);
        unsigned long long hsum = 0;
        long nsum = 0;
        MPI_Reduce(&h, &hsum, 1, MPI_UNSIGNED_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
        MPI_Reduce(&s->nrecv, &nsum, 1, MPI_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
        if (rank == 0) printf("is iteration %d keys %ld checksum %016llx\n", it, nsum, hsum);
    }
    const double t1 = MPI_Wtime();

    // full verification: place every received key at its rank, check order locally and across ranks
    const long nrecv = s->nrecv;
    long errors = 0;
    for (int c = 0; c < NCHUNK; c++) errors += s->bad[c];
    gpumpi_parallel_for(NCHUNK, place_chunk, s);
    int* sorted = s->sorted;
    for (long i = 1; i < nrecv; i++)
        if (sorted[i - 1] > sorted[i]) errors++;
    int last = nrecv > 0 ? sorted[nrecv - 1] : -1, prev_last = -1;
    // pass the largest key seen so far along the ranks, so empty ranks do not break the chain
    if (rank > 0) MPI_Recv(&prev_last, 1, MPI_INT, rank - 1, 5, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
    if (nrecv > 0 && prev_last > sorted[0]) errors++;
    if (prev_last > last) last = prev_last;
    if (rank < size - 1) MPI_Send(&last, 1, MPI_INT, rank + 1, 5, MPI_COMM_WORLD);
    unsigned long long fold = 0;
    for (long i = 0; i < nrecv; i++) fold = fold * 0x100000001B3ull + (unsigned long long)sorted[i];
    long errs = 0, keys_total = 0;
    unsigned long long fsum = 0;
    double dt = t1 - t0, tmax = 0;
    MPI_Reduce(&errors, &errs, 1, MPI_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce((void*)&nrecv, &keys_total, 1, MPI_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce(&fold, &fsum, 1, MPI_UNSIGNED_LONG_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce(&dt, &tmax, 1, MPI_DOUBLE, MPI_MAX, 0, MPI_COMM_WORLD);
    int status = 0;
    if (rank == 0) {
        printf("is verify keys %ld errors %ld sorted-checksum %016llx %s\n", keys_total, errs, fsum,
               errs == 0 && keys_total == total ? "PASSED" : "FAILED");
        printf("is-time seconds %.6f Mkeys_per_s %.3f\n", tmax, tmax > 0 ? (double)total * iters / tmax / 1e6 : 0.0);
        status = errs == 0 && keys_total == total ? 0 : 1;
    }
    free(s->keys);
    free(s->sendk);
    free(s->recvk);
    free(s->sorted);
    free(s->chist);
    free(s->bstart);
    free(s->cnt);
    free(s->bad);
    free(s->csum);
    free(s);
    free(hist);
    free(ghist);
    free(owner);
    free(scount);
    free(rcount);
    free(sdispl);
    free(rdispl);
    MPI_Finalize();
    return status;
}

__device__ int __gpu_max_threads() { return 1024; }
