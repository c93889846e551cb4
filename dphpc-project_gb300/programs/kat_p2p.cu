// Known-answer point-to-point scenarios, restating the patterns of the
// reference's tests/cuda_mpi_test.cu (single int :5-36, 16-int array :38-73,
// bidirectional exchange :75-127, repeated sizes with distinct tags :129-174,
// 3-rank ring flood :177-233, 10-rank all-to-all x20 :235-317) through the
// MPI API, plus wildcard, probe, status and rendezvous-size cases.
// Every rank prints "<scenario> rank <r> ok <0|1>".
// Usage: kat_p2p <scenario> ---gpumpi -n <ranks>
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"

__device__ int single_int(int rank) {
    int ok = 1;
    if (rank == 0) {
        int x = 3456;
        MPI_Send(&x, 1, MPI_INT, 1, 15, MPI_COMM_WORLD);
    } else if (rank == 1) {
        int x = 0;
        MPI_Recv(&x, 1, MPI_INT, 0, 15, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        ok = x == 3456;
    }
    return ok;
}

__device__ int array16(int rank) {
    int ok = 1;
    int x[16];
    if (rank == 0) {
        for (int i = 0; i < 16; i++) x[i] = i;
        MPI_Send(x, 16, MPI_INT, 1, 15, MPI_COMM_WORLD);
    } else if (rank == 1) {
        for (int i = 0; i < 16; i++) x[i] = 0;
        MPI_Recv(x, 16, MPI_INT, 0, 15, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        for (int i = 0; i < 16; i++)
            if (x[i] != i) ok = 0;
    }
    return ok;
}

__device__ int sendrecv(int rank) {
    int ok = 1;
    int x[16], y[16];
    MPI_Request req[2];
    int other = 1 - rank;
    for (int i = 0; i < 16; i++) {
        x[i] = rank == 0 ? i : -i;
        y[i] = 0;
    }
    MPI_Irecv(y, 16, MPI_INT, other, 15, MPI_COMM_WORLD, &req[0]);
    MPI_Isend(x, 16, MPI_INT, other, 15, MPI_COMM_WORLD, &req[1]);
    MPI_Wait(&req[0], MPI_STATUS_IGNORE);
    for (int i = 0; i < 16; i++)
        if (y[i] != (rank == 0 ? -i : i)) ok = 0;
    MPI_Wait(&req[1], MPI_STATUS_IGNORE);
    return ok;
}

__device__ int repeat_sizes(int rank) {
    const int reps = 5, n = 1 << (reps - 1);
    int other = (rank + 1) % 2;
    int local[16], remote[16];
    MPI_Request sreq[5], rreq[5];
    for (int i = 0; i < n; i++) {
        local[i] = (rank + 1) * i;
        remote[i] = 0;
    }
    for (int i = 0; i < reps; i++) {
        MPI_Isend(local, 1 << i, MPI_INT, other, i + 10, MPI_COMM_WORLD, &sreq[i]);
        MPI_Irecv(remote, 1 << i, MPI_INT, other, i + 10, MPI_COMM_WORLD, &rreq[i]);
    }
    for (int i = 0; i < reps; i++) {
        MPI_Wait(&sreq[i], MPI_STATUS_IGNORE);
        MPI_Wait(&rreq[i], MPI_STATUS_IGNORE);
    }
    int ok = 1;
    for (int i = 0; i < n; i++)
        if (remote[i] != (other + 1) * i) ok = 0;
    return ok;
}

__device__ int flood(int rank, int size) {
    const int reps = 5, n = 1 << (reps - 1);
    int next = (rank + 1) % size, prev = (size + rank - 1) % size;
    int local[16], pd[16], nd[16];
    MPI_Request sn[5], rn[5], sp[5], rp[5];
    for (int i = 0; i < n; i++) {
        local[i] = (rank + 1) * i;
        pd[i] = nd[i] = 0;
    }
    for (int i = 0; i < reps; i++) {
        int tag = i + 10;
        MPI_Isend(local, 1 << i, MPI_INT, next, tag, MPI_COMM_WORLD, &sn[i]);
        MPI_Irecv(nd, 1 << i, MPI_INT, next, tag, MPI_COMM_WORLD, &rn[i]);
        MPI_Isend(local, 1 << i, MPI_INT, prev, tag, MPI_COMM_WORLD, &sp[i]);
        MPI_Irecv(pd, 1 << i, MPI_INT, prev, tag, MPI_COMM_WORLD, &rp[i]);
    }
    for (int i = 0; i < reps; i++) {
        MPI_Wait(&rp[i], MPI_STATUS_IGNORE);
        MPI_Wait(&sn[i], MPI_STATUS_IGNORE);
        MPI_Wait(&sp[i], MPI_STATUS_IGNORE);
        MPI_Wait(&rn[i], MPI_STATUS_IGNORE);
    }
    int ok = 1;
    for (int i = 0; i < n; i++) {
        if (pd[i] != (prev + 1) * i) ok = 0;
        if (nd[i] != (next + 1) * i) ok = 0;
    }
    return ok;
}

__device__ int all_to_all(int rank, int size, int reps, int distinct) {
    const int n = 16;
    int* local = (int*)malloc(sizeof(int) * n * reps * size);
    int* remote = (int*)malloc(sizeof(int) * n * reps * size);
    MPI_Request* sreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * size);
    MPI_Request* rreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * size);
    MPI_Comm comm;
    int drc = MPI_Comm_dup(MPI_COMM_WORLD, &comm);
    int dsz = -1, drk = -1;
    MPI_Comm_size(comm, &dsz);
    MPI_Comm_rank(comm, &drk);
    if (drc != MPI_SUCCESS || dsz != size || drk != rank)
        printf("all_to_all rank %d: Comm_dup rc %d size %d rank %d\n", rank, drc, dsz, drk);
    for (int r = 0; r < size; r++)
        for (int k = 0; k < reps; k++)
            for (int i = 0; i < n; i++) {
                int idx = i + k * n + r * n * reps;
                local[idx] = i * k * r;
                remote[idx] = 0;
            }
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank) {
                int idx = k * n + r * n * reps;
                int tag = distinct ? 15 + k : 15;
                MPI_Isend(local + idx, n, MPI_INT, r, tag, comm, &sreq[r + k * size]);
                MPI_Irecv(remote + idx, n, MPI_INT, r, tag, comm, &rreq[r + k * size]);
            }
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank) {
                MPI_Status st;
                MPI_Wait(&sreq[r + k * size], MPI_STATUS_IGNORE);
                MPI_Wait(&rreq[r + k * size], &st);
                if (st.MPI_SOURCE != r) {
                    printf("all_to_all status rank %d from %d rep %d: source %d tag %d\n", rank, r, k,
                           st.MPI_SOURCE, st.MPI_TAG);
                }
            }
    int ok = 1;
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank)
                for (int i = 0; i < n; i++)
                    if (remote[i + k * n + r * n * reps] != i * k * rank) {
                        if (ok)
                            printf("all_to_all mismatch rank %d from %d rep %d elem %d: got %d want %d\n",
                                   rank, r, k, i, remote[i + k * n + r * n * reps], i * k * rank);
                        ok = 0;
                    }
    MPI_Comm_free(&comm);
    free(local);
    free(remote);
    free(sreq);
    free(rreq);
    return ok;
}


// Message-identity variant of all_to_all: payload = (sender, rep, receiver, ...).
__device__ int a2a_ids(int rank, int size, int reps) {
    const int n = 16;
    int* local = (int*)malloc(sizeof(int) * n * reps * size);
    int* remote = (int*)malloc(sizeof(int) * n * reps * size);
    MPI_Request* sreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * size);
    MPI_Request* rreq = (MPI_Request*)malloc(sizeof(MPI_Request) * reps * size);
    for (int r = 0; r < size; r++)
        for (int k = 0; k < reps; k++)
            for (int i = 0; i < n; i++) {
                int idx = i + k * n + r * n * reps;
                local[idx] = i == 0 ? rank : (i == 1 ? k : (i == 2 ? r : 1000 * rank + k));
                remote[idx] = -1;
            }
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank) {
                int idx = k * n + r * n * reps;
                MPI_Isend(local + idx, n, MPI_INT, r, 15, MPI_COMM_WORLD, &sreq[r + k * size]);
                MPI_Irecv(remote + idx, n, MPI_INT, r, 15, MPI_COMM_WORLD, &rreq[r + k * size]);
            }
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank) {
                MPI_Wait(&sreq[r + k * size], MPI_STATUS_IGNORE);
                MPI_Wait(&rreq[r + k * size], MPI_STATUS_IGNORE);
            }
    int ok = 1;
    for (int k = 0; k < reps; k++)
        for (int r = 0; r < size; r++)
            if (r != rank) {
                int* m = remote + k * n + r * n * reps;
                if (m[0] != r || m[1] != k || m[2] != rank || m[3] != 1000 * r + k) {
                    printf("a2a_ids rank %d slot(from %d rep %d) got (sender %d rep %d dest %d tail %d)\n", rank, r,
                           k, m[0], m[1], m[2], m[3]);
                    ok = 0;
                }
            }
    free(local);
    free(remote);
    free(sreq);
    free(rreq);
    return ok;
}

// Wildcard receives posted after the messages arrived (the reference ignored
// wildcards on arrived messages), with filled status and MPI_Get_count.
__device__ int wildcard(int rank, int size) {
    int ok = 1;
    if (rank != 0) {
        int v[3] = {rank, rank * 10, rank * 100};
        MPI_Send(v, rank % 3 + 1, MPI_INT, 0, 100 + rank, MPI_COMM_WORLD);
    }
    MPI_Barrier(MPI_COMM_WORLD);
    if (rank == 0) {
        int seen = 0;
        for (int k = 1; k < size; k++) {
            int v[3] = {0, 0, 0};
            MPI_Status st;
            MPI_Recv(v, 3, MPI_INT, MPI_ANY_SOURCE, MPI_ANY_TAG, MPI_COMM_WORLD, &st);
            int cnt = -1;
            MPI_Get_count(&st, MPI_INT, &cnt);
            int src = st.MPI_SOURCE;
            if (src < 1 || src >= size) ok = 0;
            else {
                if (st.MPI_TAG != 100 + src) ok = 0;
                if (cnt != src % 3 + 1) ok = 0;
                if (v[0] != src) ok = 0;
                if (cnt > 1 && v[1] != src * 10) ok = 0;
                seen |= 1 << src;
            }
        }
        if (seen != ((1 << size) - 2)) ok = 0;
    }
    return ok;
}

// Probe then receive a message of unknown length; non-overtaking between
// one sender and one receiver with equal tags.
__device__ int probe_order(int rank, int size) {
    int ok = 1;
    if (rank == 1) {
        for (int k = 0; k < 8; k++) {
            int* v = (int*)malloc(sizeof(int) * (k + 1));
            for (int i = 0; i <= k; i++) v[i] = k;
            MPI_Send(v, k + 1, MPI_INT, 0, 7, MPI_COMM_WORLD);
            free(v);
        }
    } else if (rank == 0) {
        for (int k = 0; k < 8; k++) {
            MPI_Status st;
            MPI_Probe(1, 7, MPI_COMM_WORLD, &st);
            int cnt = 0;
            MPI_Get_count(&st, MPI_INT, &cnt);
            if (cnt != k + 1) ok = 0;
            int* v = (int*)malloc(sizeof(int) * (cnt > 0 ? cnt : 1));
            MPI_Recv(v, cnt, MPI_INT, 1, 7, MPI_COMM_WORLD, &st);
            for (int i = 0; i < cnt; i++)
                if (v[i] != k) ok = 0;
            free(v);
        }
        int flag = 1;
        MPI_Iprobe(MPI_ANY_SOURCE, MPI_ANY_TAG, MPI_COMM_WORLD, &flag, MPI_STATUS_IGNORE);
        if (flag) ok = 0;
    }
    (void)size;
    return ok;
}

// Messages above the eager threshold (rendezvous), in both directions at
// once with Sendrecv, and a ring shift with Sendrecv_replace.
__device__ int large(int rank, int size) {
    const int n = 1 << 18;  // 1 MiB of ints
    int ok = 1;
    int* a = (int*)malloc(sizeof(int) * n);
    int* b = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; i++) {
        a[i] = rank * 1000003 + i;
        b[i] = -1;
    }
    int next = (rank + 1) % size, prev = (rank + size - 1) % size;
    MPI_Status st;
    MPI_Sendrecv(a, n, MPI_INT, next, 3, b, n, MPI_INT, prev, 3, MPI_COMM_WORLD, &st);
    for (int i = 0; i < n; i++)
        if (b[i] != prev * 1000003 + i) {
            ok = 0;
            break;
        }
    if (st.MPI_SOURCE != prev || st.MPI_TAG != 3) ok = 0;
    MPI_Sendrecv_replace(a, n, MPI_INT, next, 4, prev, 4, MPI_COMM_WORLD, &st);
    for (int i = 0; i < n; i++)
        if (a[i] != prev * 1000003 + i) {
            ok = 0;
            break;
        }
    free(a);
    free(b);
    return ok;
}

// Waitany / Waitsome / Testall over a batch of receives.
__device__ int completion(int rank, int size) {
    int ok = 1;
    const int k = 6;
    if (rank == 0) {
        int vals[6];
        MPI_Request req[6];
        for (int i = 0; i < k; i++) MPI_Irecv(&vals[i], 1, MPI_INT, 1 + i % (size - 1), i, MPI_COMM_WORLD, &req[i]);
        int done = 0, idx = -1;
        MPI_Waitany(k, req, &idx, MPI_STATUS_IGNORE);
        if (idx < 0 || idx >= k) ok = 0;
        done++;
        while (done < k) {
            int out = 0, ids[6];
            MPI_Waitsome(k, req, &out, ids, MPI_STATUSES_IGNORE);
            if (out == MPI_UNDEFINED) break;
            done += out;
        }
        int flag = 0;
        MPI_Testall(k, req, &flag, MPI_STATUSES_IGNORE);
        if (!flag || done != k) ok = 0;
        for (int i = 0; i < k; i++)
            if (vals[i] != 1000 + i) ok = 0;
    } else {
        for (int i = 0; i < k; i++)
            if (1 + i % (size - 1) == rank) {
                int v = 1000 + i;
                MPI_Send(&v, 1, MPI_INT, 0, i, MPI_COMM_WORLD);
            }
    }
    return ok;
}

// MPI_COMM_SELF: messages to oneself (eager and rendezvous sizes), the member's
// job rank through its group, a collective and a duplicate, with WORLD traffic
// of the same tag in flight.
__device__ int self_comm(int rank, int size) {
    int ok = 1, me = -1, n = -1;
    MPI_Comm_rank(MPI_COMM_SELF, &me);
    MPI_Comm_size(MPI_COMM_SELF, &n);
    if (me != 0 || n != 1) ok = 0;
    const int next = (rank + 1) % size, prev = (rank + size - 1) % size;
    int wx = 5000 + rank, wy = -1, x = 7000 + rank, y = -1;
    MPI_Request rw[2], rs;
    MPI_Irecv(&wy, 1, MPI_INT, prev, 5, MPI_COMM_WORLD, &rw[0]);
    MPI_Isend(&wx, 1, MPI_INT, next, 5, MPI_COMM_WORLD, &rw[1]);
    MPI_Isend(&x, 1, MPI_INT, 0, 5, MPI_COMM_SELF, &rs);
    MPI_Status st;
    MPI_Recv(&y, 1, MPI_INT, 0, 5, MPI_COMM_SELF, &st);
    MPI_Wait(&rs, MPI_STATUS_IGNORE);
    MPI_Waitall(2, rw, MPI_STATUSES_IGNORE);
    if (y != 7000 + rank || st.MPI_SOURCE != 0 || st.MPI_TAG != 5) ok = 0;
    if (wy != 5000 + prev) ok = 0;
    const int big = 1 << 16;
    int* a = (int*)malloc(sizeof(int) * big);
    int* b = (int*)malloc(sizeof(int) * big);
    for (int i = 0; i < big; i++) {
        a[i] = rank * 131 + i;
        b[i] = -1;
    }
    MPI_Sendrecv(a, big, MPI_INT, 0, 9, b, big, MPI_INT, 0, 9, MPI_COMM_SELF, &st);
    for (int i = 0; i < big; i++)
        if (b[i] != rank * 131 + i) {
            ok = 0;
            break;
        }
    MPI_Group gs, gw;
    MPI_Comm_group(MPI_COMM_SELF, &gs);
    MPI_Comm_group(MPI_COMM_WORLD, &gw);
    int zero = 0, wr = -1;
    MPI_Group_translate_ranks(gs, 1, &zero, gw, &wr);
    if (wr != rank) ok = 0;
    MPI_Group_free(&gs);
    MPI_Group_free(&gw);
    int sum = 0;
    MPI_Allreduce(&x, &sum, 1, MPI_INT, MPI_SUM, MPI_COMM_SELF);
    if (sum != x) ok = 0;
    MPI_Comm d;
    MPI_Comm_dup(MPI_COMM_SELF, &d);
    int dx = 9000 + rank, dy = -1;
    MPI_Sendrecv(&dx, 1, MPI_INT, 0, 1, &dy, 1, MPI_INT, 0, 1, d, MPI_STATUS_IGNORE);
    if (dy != dx) ok = 0;
    MPI_Comm_free(&d);
    free(a);
    free(b);
    return ok;
}

// Point to point on communicators from MPI_Comm_split (even and odd world
// ranks, reversed order): blocking sends and receives, Sendrecv, receives
// posted before the matching sends, rendezvous sizes and MPI_ANY_SOURCE, with
// WORLD messages of the same tags in flight.  Sources in statuses are ranks
// of the sub-communicator.
__device__ int split_p2p(int rank, int size) {
    int ok = 1, me = -1, n = -1;
    MPI_Comm sub;
    MPI_Comm_split(MPI_COMM_WORLD, rank % 2, size - rank, &sub);
    MPI_Comm_rank(sub, &me);
    MPI_Comm_size(sub, &n);
    const int next = (me + 1) % n, prev = (me + n - 1) % n;
    // a WORLD message of tag 3 to the next world rank, received at the end
    const int wnext = (rank + 1) % size, wprev = (rank + size - 1) % size;
    int wv = 100 + rank, wr = -1;
    MPI_Request wreq[2];
    MPI_Irecv(&wr, 1, MPI_INT, wprev, 3, MPI_COMM_WORLD, &wreq[0]);
    MPI_Isend(&wv, 1, MPI_INT, wnext, 3, MPI_COMM_WORLD, &wreq[1]);
    // blocking ring on sub, tag 3: even members send first
    int x = 1000 * (rank % 2) + me, y = -1;
    MPI_Status st;
    if (me % 2 == 0) {
        MPI_Send(&x, 1, MPI_INT, next, 3, sub);
        MPI_Recv(&y, 1, MPI_INT, prev, 3, sub, &st);
    } else {
        MPI_Recv(&y, 1, MPI_INT, prev, 3, sub, &st);
        MPI_Send(&x, 1, MPI_INT, next, 3, sub);
    }
    if (y != 1000 * (rank % 2) + prev || st.MPI_SOURCE != prev || st.MPI_TAG != 3) ok = 0;
    // Sendrecv of 40 doubles the other way
    double d[40], e[40];
    for (int i = 0; i < 40; i++) d[i] = rank * 0.5 + i;
    MPI_Sendrecv(d, 40, MPI_DOUBLE, prev, 4, e, 40, MPI_DOUBLE, next, 4, sub, &st);
    int wnext_sub = -1;
    {
        MPI_Group gs, gw;
        MPI_Comm_group(sub, &gs);
        MPI_Comm_group(MPI_COMM_WORLD, &gw);
        MPI_Group_translate_ranks(gs, 1, &next, gw, &wnext_sub);
        MPI_Group_free(&gs);
        MPI_Group_free(&gw);
    }
    for (int i = 0; i < 40; i++)
        if (e[i] != wnext_sub * 0.5 + i) ok = 0;
    if (st.MPI_SOURCE != next) ok = 0;
    // receives posted first, then the sends: 8 bytes and 256 KiB
    const int big = 1 << 16;
    int* a = (int*)malloc(sizeof(int) * big);
    int* b = (int*)malloc(sizeof(int) * big);
    for (int i = 0; i < big; i++) {
        a[i] = rank * 7 + i;
        b[i] = -1;
    }
    long long sv = 5000 + rank, rv = -1;
    MPI_Request rq[2];
    MPI_Irecv(&rv, 1, MPI_LONG_LONG, prev, 6, sub, &rq[0]);
    MPI_Irecv(b, big, MPI_INT, next, 7, sub, &rq[1]);
    MPI_Send(&sv, 1, MPI_LONG_LONG, next, 6, sub);
    MPI_Send(a, big, MPI_INT, prev, 7, sub);
    MPI_Waitall(2, rq, MPI_STATUSES_IGNORE);
    int wprev_sub = -1;
    {
        MPI_Group gs, gw;
        MPI_Comm_group(sub, &gs);
        MPI_Comm_group(MPI_COMM_WORLD, &gw);
        MPI_Group_translate_ranks(gs, 1, &prev, gw, &wprev_sub);
        MPI_Group_free(&gs);
        MPI_Group_free(&gw);
    }
    if (rv != 5000 + wprev_sub) ok = 0;
    for (int i = 0; i < big; i++)
        if (b[i] != wnext_sub * 7 + i) {
            ok = 0;
            break;
        }
    // member 0 gathers one value from every other member with MPI_ANY_SOURCE
    if (me == 0) {
        int seen = 0;
        for (int k = 1; k < n; k++) {
            int v = -1;
            MPI_Recv(&v, 1, MPI_INT, MPI_ANY_SOURCE, 8, sub, &st);
            if (st.MPI_SOURCE < 1 || st.MPI_SOURCE >= n || v != 300 + st.MPI_SOURCE) ok = 0;
            seen |= 1 << st.MPI_SOURCE;
        }
        if (seen != ((1 << n) - 2)) ok = 0;
    } else {
        int v = 300 + me;
        MPI_Send(&v, 1, MPI_INT, 0, 8, sub);
    }
    MPI_Waitall(2, wreq, MPI_STATUSES_IGNORE);
    if (wr != 100 + wprev) ok = 0;
    MPI_Comm_free(&sub);
    free(a);
    free(b);
    return ok;
}

// Matching follows posting order: messages already in the mailbox go to the
// earliest posted matching receive, whether it was posted by MPI_Irecv (still
// waiting) or by a later blocking MPI_Recv.
__device__ int posted_order(int rank, int size) {
    int ok = 1;
    if (rank == 1) {
        for (int i = 0; i < 4; i++) {
            int v = 10 + i;
            MPI_Send(&v, 1, MPI_INT, 0, 5, MPI_COMM_WORLD);
        }
    }
    MPI_Barrier(MPI_COMM_WORLD);   // the eager messages are in rank 0's mailbox
    if (rank == 0) {
        int a = -1, b = -1, c = -1, d = -1;
        MPI_Request ra, rc;
        MPI_Status st;
        MPI_Irecv(&a, 1, MPI_INT, MPI_ANY_SOURCE, 5, MPI_COMM_WORLD, &ra);
        MPI_Recv(&b, 1, MPI_INT, 1, 5, MPI_COMM_WORLD, &st);
        MPI_Irecv(&c, 1, MPI_INT, 1, MPI_ANY_TAG, MPI_COMM_WORLD, &rc);
        MPI_Sendrecv(&a, 0, MPI_INT, 0, 9, &d, 1, MPI_INT, 1, 5, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        MPI_Wait(&rc, MPI_STATUS_IGNORE);
        MPI_Wait(&ra, MPI_STATUS_IGNORE);
        int z = -1;
        MPI_Recv(&z, 0, MPI_INT, 0, 9, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        ok = a == 10 && b == 11 && c == 12 && d == 13 && st.MPI_SOURCE == 1;
    }
    MPI_Barrier(MPI_COMM_WORLD);
    return ok;
}

// Streams of tiny blocking messages (1..16 bytes, odd buffer offsets) from
// every other rank to rank 0, more than a mailbox holds, received with
// MPI_ANY_SOURCE / MPI_ANY_TAG: per sender in send order, with the right
// size, tag and bytes.
__device__ unsigned char tiny_byte(int src, int k, int j) { return (unsigned char)((src * 31 + k * 7 + j * 13) & 0xff); }
__device__ int tiny_len(int src, int k) { return 1 + (k * 7 + src) % 16; }

__device__ int tiny_stream(int rank, int size) {
    const int n = 200;
    int ok = 1;
    unsigned char buf[40];
    if (rank > 0) {
        for (int k = 0; k < n; k++) {
            unsigned char* p = buf + 1 + k % 3;
            const int len = tiny_len(rank, k);
            for (int j = 0; j < len; j++) p[j] = tiny_byte(rank, k, j);
            if (MPI_Send(p, len, MPI_BYTE, 0, k % 4, MPI_COMM_WORLD) != MPI_SUCCESS) ok = 0;
        }
    } else {
        int next[64];
        for (int r = 0; r < size && r < 64; r++) next[r] = 0;
        for (int m = 0; m < n * (size - 1); m++) {
            unsigned char* p = buf + 3 + m % 5;
            MPI_Status st;
            if (MPI_Recv(p, 16, MPI_BYTE, MPI_ANY_SOURCE, MPI_ANY_TAG, MPI_COMM_WORLD, &st) != MPI_SUCCESS) ok = 0;
            const int src = st.MPI_SOURCE;
            if (src < 1 || src >= size || src >= 64) {
                ok = 0;
                continue;
            }
            const int k = next[src]++;
            int cnt = -1;
            MPI_Get_count(&st, MPI_BYTE, &cnt);
            if (cnt != tiny_len(src, k) || st.MPI_TAG != k % 4) ok = 0;
            for (int j = 0; j < cnt && j < 16; j++)
                if (p[j] != tiny_byte(src, k, j)) ok = 0;
        }
        for (int r = 1; r < size && r < 64; r++)
            if (next[r] != n) ok = 0;
    }
    MPI_Barrier(MPI_COMM_WORLD);
    return ok;
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size, ok = 0;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const char* s = argc > 1 ? argv[1] : "single_int";
    if (!strcmp(s, "single_int")) ok = single_int(rank);
    else if (!strcmp(s, "array16")) ok = array16(rank);
    else if (!strcmp(s, "sendrecv")) ok = sendrecv(rank);
    else if (!strcmp(s, "repeat_sizes")) ok = repeat_sizes(rank);
    else if (!strcmp(s, "flood")) ok = flood(rank, size);
    else if (!strcmp(s, "all_to_all"))
        ok = all_to_all(rank, size, argc > 2 ? atoi(argv[2]) : 20, argc > 3 ? atoi(argv[3]) : 0);
    else if (!strcmp(s, "a2a_ids")) ok = a2a_ids(rank, size, argc > 2 ? atoi(argv[2]) : 3);
    else if (!strcmp(s, "wildcard")) ok = wildcard(rank, size);
    else if (!strcmp(s, "probe_order")) ok = probe_order(rank, size);
    else if (!strcmp(s, "large")) ok = large(rank, size);
    else if (!strcmp(s, "completion")) ok = completion(rank, size);
    else if (!strcmp(s, "self_comm")) ok = self_comm(rank, size);
    else if (!strcmp(s, "split_p2p")) ok = split_p2p(rank, size);
    else if (!strcmp(s, "posted_order")) ok = posted_order(rank, size);
    else if (!strcmp(s, "tiny_stream")) ok = tiny_stream(rank, size);
    printf("%s rank %d ok %d\n", s, rank, ok);
    MPI_Finalize();
    return 0;
}

__device__ int __gpu_max_threads() { return 1024; }
