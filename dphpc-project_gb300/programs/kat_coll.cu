// Known-answer collective and communicator scenarios, restating the reference's
// tests/collectives_test.cu (Reduce PROD int16 on 5 ranks :6-54, Allreduce SUM
// double on 7 :57-98, Allgather 7 :100-141, Scatter from root 2 :144-196,
// Scatterv sizes i+1 :199-288) and tests/communicator_test.cu (rank equals
// launch rank :5-25, three Comm_dup contexts with crossed traffic :27-90,
// Comm_split colors/keys :93-152), plus closed-form checks of the collectives
// the reference lacks or stubs.  Every rank prints "<scenario> rank <r> ok <0|1>".
// Usage: kat_coll <scenario> ---gpumpi -n <ranks>
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "stdint.h.cuh"
#include "omp.h.cuh"

__device__ int reduce_prod(int rank, int size) {
    int16_t buf[14], out[14], expect[14];
    for (int i = 0; i < 14; i++) {
        buf[i] = (int16_t)((rank + 1) * (i + 1));
        out[i] = 0;
        expect[i] = 1;
    }
    for (int r = 0; r < size; r++)
        for (int i = 0; i < 14; i++) expect[i] = (int16_t)(expect[i] * (r + 1) * (i + 1));
    MPI_Reduce(buf, out, 14, MPI_INT16_T, MPI_PROD, 0, MPI_COMM_WORLD);
    int ok = 1;
    if (rank == 0)
        for (int i = 0; i < 14; i++)
            if (out[i] != expect[i]) ok = 0;
    return ok;
}

__device__ int allreduce_sum(int rank, int size) {
    double buf[17], out[17], expect[17];
    for (int i = 0; i < 17; i++) {
        buf[i] = (rank + 1) * (i + 1);
        out[i] = 0;
        expect[i] = 0;
    }
    for (int r = 0; r < size; r++)
        for (int i = 0; i < 17; i++) expect[i] += (r + 1) * (i + 1);
    MPI_Allreduce(buf, out, 17, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
    int ok = 1;
    for (int i = 0; i < 17; i++)
        if (out[i] != expect[i]) ok = 0;
    return ok;
}

__device__ int allgather(int rank, int size) {
    const int n = 7;
    int* buf = (int*)malloc(sizeof(int) * n);
    int* out = (int*)malloc(sizeof(int) * n * size);
    for (int i = 0; i < n; i++) buf[i] = (rank + 1) * (i + 1);
    MPI_Allgather(buf, n, MPI_INT, out, n, MPI_INT, MPI_COMM_WORLD);
    int ok = 1;
    for (int r = 0; r < size; r++)
        for (int i = 0; i < n; i++)
            if (out[r * n + i] != (r + 1) * (i + 1)) ok = 0;
    free(buf);
    free(out);
    return ok;
}

__device__ int scatter(int rank, int size) {
    const int root = 2, n = 4;
    int* sb = (int*)malloc(sizeof(int) * n * size);
    int rb[4];
    for (int j = 0; j < size; j++)
        for (int i = 0; i < n; i++) sb[i + j * n] = rank == root ? j : -2;
    for (int i = 0; i < n; i++) rb[i] = -1;
    MPI_Scatter(sb, n, MPI_INT, rb, n, MPI_INT, root, MPI_COMM_WORLD);
    int ok = 1;
    for (int i = 0; i < n; i++)
        if (rb[i] != rank) ok = 0;
    free(sb);
    return ok;
}

__device__ int scatterv(int rank, int size) {
    const int root = 2;
    int* sizes = (int*)malloc(sizeof(int) * size);
    int* displs = (int*)malloc(sizeof(int) * size);
    for (int i = 0; i < size; i++) {
        sizes[i] = i + 1;
        displs[i] = i == 0 ? 0 : displs[i - 1] + sizes[i - 1];
    }
    int total = displs[size - 1] + sizes[size - 1];
    int* sb = (int*)malloc(sizeof(int) * total);
    int* rb = (int*)malloc(sizeof(int) * sizes[rank]);
    for (int j = 0; j < size; j++)
        for (int i = 0; i < sizes[j]; i++) sb[displs[j] + i] = rank == root ? j : -2;
    for (int i = 0; i < sizes[rank]; i++) rb[i] = -1;
    MPI_Scatterv(sb, sizes, displs, MPI_INT, rb, sizes[rank], MPI_INT, root, MPI_COMM_WORLD);
    int ok = 1;
    for (int i = 0; i < sizes[rank]; i++)
        if (rb[i] != rank) ok = 0;
    free(sizes);
    free(displs);
    free(sb);
    free(rb);
    return ok;
}

__device__ int comm_rank(int rank, int size) {
    int r = -1, s = -1;
    MPI_Comm_rank(MPI_COMM_WORLD, &r);
    MPI_Comm_size(MPI_COMM_WORLD, &s);
    return r == rank && s == size;
}

__device__ int comm_dup_traffic(int rank, int size) {
    (void)size;
    MPI_Comm c1, c2, c3;
    MPI_Comm_dup(MPI_COMM_WORLD, &c1);
    MPI_Comm_dup(MPI_COMM_WORLD, &c2);
    MPI_Comm_dup(c2, &c3);
    MPI_Request req[3];
    int16_t data[30];
    int ok = 1;
    if (rank == 0) {
        for (int i = 0; i < 30; i++) data[i] = (int16_t)(i + 1);
        MPI_Isend(data + 0, 10, MPI_INT16_T, 1, 17, c1, &req[0]);
        MPI_Irecv(data + 10, 10, MPI_INT16_T, 1, 17, c2, &req[1]);
        MPI_Isend(data + 20, 10, MPI_INT16_T, 1, 17, c3, &req[2]);
    } else if (rank == 1) {
        for (int i = 0; i < 30; i++) data[i] = (int16_t)(-(i + 1));
        MPI_Irecv(data + 20, 10, MPI_INT16_T, 0, 17, c3, &req[2]);
        MPI_Irecv(data + 0, 10, MPI_INT16_T, 0, 17, c1, &req[0]);
        MPI_Isend(data + 10, 10, MPI_INT16_T, 0, 17, c2, &req[1]);
    }
    if (rank <= 1) {
        MPI_Status st[3];
        MPI_Waitall(3, req, st);
    }
    if (rank == 0) {
        for (int i = 10; i < 20; i++)
            if (data[i] != -(i + 1)) ok = 0;
    } else if (rank == 1) {
        for (int i = 0; i < 10; i++)
            if (data[i] != i + 1) ok = 0;
        for (int i = 20; i < 30; i++)
            if (data[i] != i + 1) ok = 0;
    }
    MPI_Comm_free(&c1);
    MPI_Comm_free(&c2);
    MPI_Comm_free(&c3);
    return ok;
}

__device__ int comm_split(int rank, int size) {
    (void)size;
    int color, key;
    if (rank < 3) {
        color = 0;
        key = rank;
    } else if (rank < 6) {
        color = 1;
        key = 6 - rank;
    } else if (rank < 9) {
        color = 2;
        key = 1;
    } else {
        color = 2;
        key = 0;
    }
    MPI_Comm c;
    MPI_Comm_split(MPI_COMM_WORLD, color, key, &c);
    int nr = -1, ns = -1;
    MPI_Comm_rank(c, &nr);
    MPI_Comm_size(c, &ns);
    int ok = 1;
    if (rank < 3) ok = nr == rank && ns == 3;
    else if (rank < 6) ok = nr == 5 - rank && ns == 3;
    else if (rank < 9) ok = nr == rank - 5 && ns == 4;
    else ok = nr == 0 && ns == 4;
    // the new communicator carries traffic and collectives of its own
    int sum = 0, one = nr + 1;
    MPI_Allreduce(&one, &sum, 1, MPI_INT, MPI_SUM, c);
    if (sum != ns * (ns + 1) / 2) ok = 0;
    MPI_Barrier(c);
    MPI_Comm_free(&c);
    return ok;
}

// Closed forms for the collectives the reference stubs or lacks.
__device__ int extras(int rank, int size) {
    int ok = 1;
    // Bcast from the last rank, local scalar buffer
    int v = rank == size - 1 ? 4242 : 0;
    MPI_Bcast(&v, 1, MPI_INT, size - 1, MPI_COMM_WORLD);
    if (v != 4242) ok = 0;
    // Gatherv to root 1
    int* counts = (int*)malloc(sizeof(int) * size);
    int* displs = (int*)malloc(sizeof(int) * size);
    int tot = 0;
    for (int q = 0; q < size; q++) {
        counts[q] = q % 3 + 1;
        displs[q] = tot;
        tot += counts[q];
    }
    int mine[3] = {rank, rank, rank};
    int* g = (int*)malloc(sizeof(int) * tot);
    MPI_Gatherv(mine, counts[rank], MPI_INT, g, counts, displs, MPI_INT, 1 % size, MPI_COMM_WORLD);
    if (rank == 1 % size)
        for (int q = 0; q < size; q++)
            for (int i = 0; i < counts[q]; i++)
                if (g[displs[q] + i] != q) ok = 0;
    // Allgatherv
    for (int i = 0; i < tot; i++) g[i] = -1;
    MPI_Allgatherv(mine, counts[rank], MPI_INT, g, counts, displs, MPI_INT, MPI_COMM_WORLD);
    for (int q = 0; q < size; q++)
        for (int i = 0; i < counts[q]; i++)
            if (g[displs[q] + i] != q) ok = 0;
    // Alltoall: element for peer q is rank*100+q
    int* a = (int*)malloc(sizeof(int) * size);
    int* b = (int*)malloc(sizeof(int) * size);
    for (int q = 0; q < size; q++) a[q] = rank * 100 + q;
    MPI_Alltoall(a, 1, MPI_INT, b, 1, MPI_INT, MPI_COMM_WORLD);
    for (int q = 0; q < size; q++)
        if (b[q] != q * 100 + rank) ok = 0;
    // Alltoallv with ragged blocks: rank sends (q+1) copies of rank to q
    int* sc = (int*)malloc(sizeof(int) * size);
    int* sd = (int*)malloc(sizeof(int) * size);
    int* rc = (int*)malloc(sizeof(int) * size);
    int* rd = (int*)malloc(sizeof(int) * size);
    int st = 0, rt = 0;
    for (int q = 0; q < size; q++) {
        sc[q] = q + 1;
        sd[q] = st;
        st += sc[q];
        rc[q] = rank + 1;
        rd[q] = rt;
        rt += rc[q];
    }
    int* sbuf = (int*)malloc(sizeof(int) * st);
    int* rbuf = (int*)malloc(sizeof(int) * rt);
    for (int i = 0; i < st; i++) sbuf[i] = rank;
    MPI_Alltoallv(sbuf, sc, sd, MPI_INT, rbuf, rc, rd, MPI_INT, MPI_COMM_WORLD);
    for (int q = 0; q < size; q++)
        for (int i = 0; i < rc[q]; i++)
            if (rbuf[rd[q] + i] != q) ok = 0;
    // Scan / Exscan of rank+1
    int s = 0, e = -7, x = rank + 1;
    MPI_Scan(&x, &s, 1, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
    if (s != (rank + 1) * (rank + 2) / 2) ok = 0;
    MPI_Exscan(&x, &e, 1, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
    if (rank > 0 && e != rank * (rank + 1) / 2) ok = 0;
    // Reduce_scatter_block: every rank contributes q+rank for block q
    int* rs = (int*)malloc(sizeof(int) * size);
    for (int q = 0; q < size; q++) rs[q] = q + rank;
    int got = 0;
    MPI_Reduce_scatter_block(rs, &got, 1, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
    if (got != size * rank + size * (size - 1) / 2) ok = 0;
    // MAXLOC / MINLOC on (value, rank) pairs
    struct {
        double val;
        int idx;
    } in, mx, mn;
    in.val = (double)((rank * 7) % size);
    in.idx = rank;
    MPI_Allreduce(&in, &mx, 1, MPI_DOUBLE_INT, MPI_MAXLOC, MPI_COMM_WORLD);
    MPI_Allreduce(&in, &mn, 1, MPI_DOUBLE_INT, MPI_MINLOC, MPI_COMM_WORLD);
    double best = -1, worst = 1e30;
    int bi = -1, wi = -1;
    for (int q = 0; q < size; q++) {
        double val = (double)((q * 7) % size);
        if (val > best) {
            best = val;
            bi = q;
        }
        if (val < worst) {
            worst = val;
            wi = q;
        }
    }
    if (mx.val != best || mx.idx != bi || mn.val != worst || mn.idx != wi) ok = 0;
    // In-place allreduce and a derived contiguous type
    int iv[2] = {rank, 1};
    MPI_Allreduce(MPI_IN_PLACE, iv, 2, MPI_INT, MPI_SUM, MPI_COMM_WORLD);
    if (iv[0] != size * (size - 1) / 2 || iv[1] != size) ok = 0;
    MPI_Datatype pair;
    MPI_Type_contiguous(2, MPI_INT, &pair);
    MPI_Type_commit(&pair);
    int tsz = 0;
    MPI_Type_size(pair, &tsz);
    if (tsz != 8) ok = 0;
    int pv[2] = {rank, 2 * rank}, po[2] = {0, 0};
    MPI_Allreduce(pv, po, 1, pair, MPI_MAX, MPI_COMM_WORLD);
    if (po[0] != size - 1 || po[1] != 2 * (size - 1)) ok = 0;
    MPI_Type_free(&pair);
    free(counts);
    free(displs);
    free(g);
    free(a);
    free(b);
    free(sc);
    free(sd);
    free(rc);
    free(rd);
    free(sbuf);
    free(rbuf);
    free(rs);
    return ok;
}

// Groups, Comm_create and Cartesian topologies.
__device__ int groups_cart(int rank, int size) {
    int ok = 1;
    MPI_Group world, evens;
    MPI_Comm_group(MPI_COMM_WORLD, &world);
    int ranges[1][3] = {{0, size - 1, 2}};
    MPI_Group_range_incl(world, 1, ranges, &evens);
    int gs = -1, gr = -2;
    MPI_Group_size(evens, &gs);
    MPI_Group_rank(evens, &gr);
    if (gs != (size + 1) / 2) ok = 0;
    if (rank % 2 == 0 && gr != rank / 2) ok = 0;
    if (rank % 2 == 1 && gr != MPI_UNDEFINED) ok = 0;
    MPI_Comm ce;
    MPI_Comm_create(MPI_COMM_WORLD, evens, &ce);
    if (rank % 2 == 0) {
        int r = -1;
        MPI_Comm_rank(ce, &r);
        if (r != rank / 2) ok = 0;
        int t = 1, sum = 0;
        MPI_Allreduce(&t, &sum, 1, MPI_INT, MPI_SUM, ce);
        if (sum != gs) ok = 0;
        MPI_Comm_free(&ce);
    } else if (ce != MPI_COMM_NULL) {
        ok = 0;
    }
    MPI_Group_free(&evens);
    MPI_Group_free(&world);
    int dims[2] = {0, 0}, periods[2] = {1, 0};
    MPI_Dims_create(size, 2, dims);
    if (dims[0] * dims[1] != size || dims[0] < dims[1]) ok = 0;
    MPI_Comm cart;
    MPI_Cart_create(MPI_COMM_WORLD, 2, dims, periods, 0, &cart);
    int cr = -1, coords[2] = {-1, -1};
    MPI_Comm_rank(cart, &cr);
    MPI_Cart_coords(cart, cr, 2, coords);
    if (coords[0] != cr / dims[1] || coords[1] != cr % dims[1]) ok = 0;
    int src = -5, dst = -5;
    MPI_Cart_shift(cart, 0, 1, &src, &dst);
    int exp_dst = ((coords[0] + 1) % dims[0]) * dims[1] + coords[1];
    if (dst != exp_dst) ok = 0;
    MPI_Cart_shift(cart, 1, 1, &src, &dst);
    if (coords[1] == dims[1] - 1 && dst != MPI_PROC_NULL) ok = 0;
    if (coords[1] < dims[1] - 1 && dst != cr + 1) ok = 0;
    int remain[2] = {0, 1};
    MPI_Comm row;
    MPI_Cart_sub(cart, remain, &row);
    int rr = -1, rsz = -1;
    MPI_Comm_rank(row, &rr);
    MPI_Comm_size(row, &rsz);
    if (rr != coords[1] || rsz != dims[1]) ok = 0;
    MPI_Comm_free(&row);
    MPI_Comm_free(&cart);
    return ok;
}

// User-defined operator that is not commutative: inout = inout * 31 + in (mod
// 2^32).  Folded in rank order (acc = x_0; acc = op(x_q, acc)) the result is
// the Horner value of x_0, x_1, ..., x_{P-1}, so any other order shows.
__device__ void horner_op(void* in, void* inout, int* len, MPI_Datatype* dt) {
    const unsigned* a = (const unsigned*)in;
    unsigned* b = (unsigned*)inout;
    for (int i = 0; i < *len; i++) b[i] = b[i] * 31u + a[i];
}

__device__ unsigned user_x(int q, long i) { return (unsigned)(q * 2654435761u) ^ (unsigned)(i * 40503u + 7u); }

__device__ int user_op(int rank, int size) {
    MPI_Op op;
    int ok = 1;
    if (MPI_Op_create(horner_op, 0, &op) != MPI_SUCCESS) return 0;
    const int counts[3] = {1, 1000, 70001};
    for (int k = 0; k < 3; k++) {
        const int n = counts[k];
        unsigned* x = (unsigned*)malloc(sizeof(unsigned) * n);
        unsigned* r = (unsigned*)malloc(sizeof(unsigned) * n);
        unsigned* a = (unsigned*)malloc(sizeof(unsigned) * n);
        for (long i = 0; i < n; i++) {
            x[i] = user_x(rank, i);
            r[i] = 0;
            a[i] = 0;
        }
        MPI_Reduce(x, r, n, MPI_UNSIGNED, op, 0, MPI_COMM_WORLD);
        MPI_Allreduce(x, a, n, MPI_UNSIGNED, op, MPI_COMM_WORLD);
        for (long i = 0; i < n; i++) {
            unsigned acc = user_x(0, i);
            for (int q = 1; q < size; q++) acc = acc * 31u + user_x(q, i);
            if (a[i] != acc) ok = 0;
            if (rank == 0 && r[i] != acc) ok = 0;
        }
        free(x);
        free(r);
        free(a);
    }
    MPI_Op_free(&op);
    if (op != MPI_OP_NULL) ok = 0;
    return ok;
}

// Parallel loop: every iteration runs once; with a rank made of several
// thread blocks (a cluster), iterations run on all of them.
struct loop_arg {
    long* out;
    int* blk;
};

__device__ void loop_body(long i, void* p) {
    struct loop_arg* a = (struct loop_arg*)p;
    a->out[i] += i * 3 + 1;
    a->blk[i] = gpumpi_loop_block();
}

__device__ int parfor(int rank, int size) {
    const long n = 200003;
    struct loop_arg* a = (struct loop_arg*)malloc(sizeof(struct loop_arg));
    a->out = (long*)malloc(sizeof(long) * n);
    a->blk = (int*)malloc(sizeof(int) * n);
    for (long i = 0; i < n; i++) {
        a->out[i] = rank;
        a->blk[i] = -1;
    }
    gpumpi_parallel_for(n, loop_body, a);
    int ok = 1;
    int seen[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (long i = 0; i < n; i++) {
        if (a->out[i] != rank + i * 3 + 1) ok = 0;
        if (a->blk[i] < 0 || a->blk[i] >= 8) ok = 0;
        else seen[a->blk[i]] = 1;
    }
    int blocks = 0;
    for (int k = 0; k < 8; k++) blocks += seen[k];
    printf("parfor rank %d blocks %d\n", rank, blocks);
    free(a->out);
    free(a->blk);
    free(a);
    return ok;
}

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size, ok = 0;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const char* s = argc > 1 ? argv[1] : "extras";
    if (!strcmp(s, "reduce_prod")) ok = reduce_prod(rank, size);
    else if (!strcmp(s, "allreduce_sum")) ok = allreduce_sum(rank, size);
    else if (!strcmp(s, "allgather")) ok = allgather(rank, size);
    else if (!strcmp(s, "scatter")) ok = scatter(rank, size);
    else if (!strcmp(s, "scatterv")) ok = scatterv(rank, size);
    else if (!strcmp(s, "comm_rank")) ok = comm_rank(rank, size);
    else if (!strcmp(s, "comm_dup_traffic")) ok = comm_dup_traffic(rank, size);
    else if (!strcmp(s, "comm_split")) ok = comm_split(rank, size);
    else if (!strcmp(s, "extras")) ok = extras(rank, size);
    else if (!strcmp(s, "groups_cart")) ok = groups_cart(rank, size);
    else if (!strcmp(s, "user_op")) ok = user_op(rank, size);
    else if (!strcmp(s, "parfor")) ok = parfor(rank, size);
    printf("%s rank %d ok %d\n", s, rank, ok);
    MPI_Finalize();
    return 0;
}

__device__ int __gpu_max_threads() { return 1024; }
