/* Converter test program: nonblocking ring exchanges into global buffers, a
 * blocking send/receive pair, and rank-order reductions.  Rank 0 prints the
 * results; the output is the same on any MPI whose reductions fold in rank
 * order. */
#include <stdio.h>
#include <mpi.h>

#define N 64
#define ITERS 10

double buf_out[N], buf_in[N];
long checks[ITERS];

int main(int argc, char *argv[])
{
    int rank, size, left, right, iter, i;
    MPI_Request req[2];
    MPI_Status st[2];
    double local = 0.0, global = 0.0;
    long lsum = 0, gsum = 0, gmax = 0;
    int token = 0;

    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    left = (rank + size - 1) % size;
    right = (rank + 1) % size;

    for (iter = 0; iter < ITERS; iter++) {
        for (i = 0; i < N; i++)
            buf_out[i] = rank * 1000.0 + iter * N + i + 0.125;
        MPI_Irecv(buf_in, N, MPI_DOUBLE, left, iter, MPI_COMM_WORLD, &req[0]);
        MPI_Isend(buf_out, N, MPI_DOUBLE, right, iter, MPI_COMM_WORLD, &req[1]);
        MPI_Waitall(2, req, st);
        checks[iter] = (long)buf_in[N - 1] + st[0].MPI_SOURCE;
        for (i = 0; i < N; i++)
            local += buf_in[i] / (i + 1);
    }
    for (iter = 0; iter < ITERS; iter++)
        lsum += checks[iter] * (iter + 1);

    /* a token passed once around the ring with blocking calls */
    if (size > 1) {
        if (rank == 0) {
            token = 1;
            MPI_Send(&token, 1, MPI_INT, right, 99, MPI_COMM_WORLD);
            MPI_Recv(&token, 1, MPI_INT, left, 99, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        } else {
            MPI_Recv(&token, 1, MPI_INT, left, 99, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
            token = token * 3 + rank;
            MPI_Send(&token, 1, MPI_INT, right, 99, MPI_COMM_WORLD);
        }
    }

    MPI_Allreduce(&local, &global, 1, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
    MPI_Reduce(&lsum, &gsum, 1, MPI_LONG, MPI_SUM, 0, MPI_COMM_WORLD);
    MPI_Reduce(&lsum, &gmax, 1, MPI_LONG, MPI_MAX, 0, MPI_COMM_WORLD);
    if (rank == 0)
        printf("ring ranks %d checksum %.10e sum %ld max %ld token %d\n", size, global, gsum, gmax, token);
    MPI_Finalize();
    return 0;
}
