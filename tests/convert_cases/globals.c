/* Converter test program: per-rank state in file-scope and function-static
 * variables, shadowing, a macro over a global, an old-style definition, the
 * implicit void* conversions C allows, and a C++ keyword used as a name.
 * Rank 0 prints one line per rank; the output is the same on any MPI. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <mpi.h>

#define NSLOT 4
#define NVAL 9
#define COUNTER_PLUS(r) (counter + (r))

struct cell {
    int id;
    double *vals;
    struct cell *next;
};

extern int counter;
int counter = 7;
static double weights[] = {0.5, 0.25, 0.125};
const int limits[3] = {10, 20, 30};
int *cursor = &counter;
char tag[] = "rank";
int grid[2][NSLOT] = {{1, 2, 3, 4}, {5, 6, 7, 8}};
struct cell head = {42, NULL, NULL};
double *scratch;
int class = 3;
int (*pick)(int);

static int twice(int x) { return 2 * x; }

int scale(a, b)
    int a;
    double b;
{
    return (int)(a * b);
}

int bump(void)
{
    static int calls = 0;
    static int hist[4] = {0};
    calls++;
    hist[calls % 4] += calls;
    return calls * 100 + hist[calls % 4];
}

double *fill(int n, double v)
{
    double *p;
    int i;
    p = malloc(n * sizeof(double));
    for (i = 0; i < n; i++)
        p[i] = v + i;
    return p;
}

double *alloc_doubles(int n) { return malloc(n * sizeof(double)); }

double sum(const double *p, int n)
{
    double s = 0;
    int i;
    for (i = 0; i < n; i++)
        s += p[i];
    return s;
}

int main(int argc, char **argv)
{
    int rank, size, i, shadowed, b;
    double row[NVAL];
    double *all = NULL;
    struct cell *c;

    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);

    counter += rank;
    grid[1][rank % NSLOT] += rank;
    class = class * (rank + 1);
    pick = twice;
    tag[0] = 'A' + rank % 26;
    scratch = fill(5, rank);
    c = malloc(sizeof *c);
    c->vals = alloc_doubles(3);
    for (i = 0; i < 3; i++)
        c->vals[i] = weights[i] * (rank + 1);
    c->id = head.id + rank;
    c->next = &head;
    {
        int counter = 1000;
        shadowed = counter + rank;
    }
    for (int k = 0; k < 2; k++) {
        int grid = k * 10;
        shadowed += grid;
    }
    bump();
    b = bump();

    /* every rank has changed its own copies before any rank reads them */
    MPI_Barrier(MPI_COMM_WORLD);

    row[0] = counter;
    row[1] = grid[1][rank % NSLOT] + grid[0][3];
    row[2] = class;
    row[3] = sum(scratch, 5) + sum(c->vals, 3);
    row[4] = *cursor + COUNTER_PLUS(1);
    row[5] = scale(rank + 3, 1.5) + pick(rank) + limits[rank % 3];
    row[6] = shadowed;
    row[7] = b;
    row[8] = strlen(tag) * 1000 + tag[0] + c->next->id;

    if (rank == 0)
        all = malloc(size * NVAL * sizeof(double));
    MPI_Gather(row, NVAL, MPI_DOUBLE, all, NVAL, MPI_DOUBLE, 0, MPI_COMM_WORLD);
    if (rank == 0) {
        for (i = 0; i < size; i++) {
            int j;
            printf("rank %d:", i);
            for (j = 0; j < NVAL; j++)
                printf(" %.4f", all[i * NVAL + j]);
            printf("\n");
        }
        free(all);
    }
    free(c->vals);
    free(c);
    free(scratch);
    MPI_Finalize();
    return 0;
}
