/* Converter test program for the allocator-version rewrites: allocations and
 * MPI_Alltoall calls made unconditionally (which get the coalescing flag),
 * conditionally (which do not), and through helper functions. */
#include <stdio.h>
#include <stdlib.h>
#include <mpi.h>

int *make(int n);

int *make(int n)
{
    int *p = malloc(n * sizeof(int));
    int i;
    for (i = 0; i < n; i++)
        p[i] = i * i;
    return p;
}

int *maybe(int n)
{
    if (n > 0)
        return malloc(n * sizeof(int));
    return NULL;
}

void exchange(int *send, int *recv, int n)
{
    MPI_Alltoall(send, n, MPI_INT, recv, n, MPI_INT, MPI_COMM_WORLD);
}

int total(int n)
{
    int *p = make(n);
    int s = 0, i;
    for (i = 0; i < n; i++)
        s += p[i];
    free(p);
    return s;
}

int main(int argc, char **argv)
{
    int rank, size, i, local, all;
    int *send, *recv, *m;

    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    send = malloc(size * 4 * sizeof(int));
    recv = malloc(size * 4 * sizeof(int));
    for (i = 0; i < size * 4; i++)
        send[i] = rank * 100 + i;
    exchange(send, recv, 4);
    local = total(rank + 3);
    for (i = 0; i < size * 4; i++)
        local += recv[i] * (i % 7);
    m = maybe(rank);
    if (m) {
        m[0] = rank;
        local += m[0];
        free(m);
    }
    MPI_Reduce(&local, &all, 1, MPI_INT, MPI_SUM, 0, MPI_COMM_WORLD);
    if (rank == 0)
        printf("coalesce ranks %d total %d\n", size, all);
    free(send);
    free(recv);
    MPI_Finalize();
    return 0;
}
