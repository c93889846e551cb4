/* Converter test program for file I/O: every rank writes a file with
 * fprintf, fputs, fputc and fwrite, reads it back with fgets, fgetc and fread,
 * seeks, and after a barrier rank 0 reads every rank's file.  Files are
 * created in the working directory and removed at the end.  Rank 0 prints
 * one line per rank; the output is the same on any MPI. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <errno.h>
#include <mpi.h>

#define NV 7

int main(int argc, char **argv)
{
    int rank, size, i;
    char name[64], line[160];
    long row[NV];
    long *all = NULL;
    FILE *f;

    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    sprintf(name, "fileio_rank%d.txt", rank);

    f = fopen(name, "w");
    if (!f) {
        printf("rank %d: cannot create %s\n", rank, name);
        MPI_Abort(MPI_COMM_WORLD, 1);
    }
    for (i = 0; i < 60 + 7 * rank; i++)
        fprintf(f, "line %d of rank %d value %.3f\n", i, rank, i * 0.5 + rank);
    fputs("tail\n", f);
    fputc('#', f);
    fputc('\n', f);
    {
        double arr[16];
        for (i = 0; i < 16; i++)
            arr[i] = rank * 100.0 + i / 8.0;
        fwrite(arr, sizeof(double), 16, f);
    }
    fclose(f);

    f = fopen(name, "r");
    {
        long lines = 0, chars = 0;
        double back[16], bsum = 0.0;
        size_t got;
        int hash, eof_before, extra, eof_after, first;
        long end_pos;
        while (fgets(line, sizeof line, f)) {
            lines++;
            chars += (long)strlen(line);
            if (strncmp(line, "tail", 4) == 0)
                break;
        }
        hash = fgetc(f);
        fgetc(f);
        got = fread(back, sizeof(double), 16, f);
        for (i = 0; i < (int)got; i++)
            bsum += back[i];
        eof_before = feof(f);
        extra = fgetc(f);
        eof_after = feof(f);
        end_pos = ftell(f);
        fseek(f, 5, SEEK_SET);
        fgets(line, sizeof line, f);
        rewind(f);
        first = fgetc(f);
        fclose(f);
        row[0] = lines;
        row[1] = chars;
        row[2] = hash + 1000 * (long)got;
        row[3] = (long)(bsum * 8.0);
        row[4] = eof_before * 100 + (extra == EOF) * 10 + eof_after;
        row[5] = end_pos;
        row[6] = first * 1000 + (long)strlen(line);
    }
    {
        FILE *m = fopen("no_such_dir/missing.txt", "r");
        row[6] += (m == NULL && errno == ENOENT) ? 1000000 : 0;
    }

    MPI_Barrier(MPI_COMM_WORLD);
    if (rank == 0) {
        /* every rank's file, written by that rank, read here */
        long total = 0;
        int q;
        for (q = 0; q < size; q++) {
            char other[64];
            long n = 0;
            sprintf(other, "fileio_rank%d.txt", q);
            f = fopen(other, "r");
            if (!f)
                continue;
            while (fgets(line, sizeof line, f))
                n++;
            fclose(f);
            total += n * (q + 1);
        }
        printf("rank 0 read all files: %ld\n", total);
        all = (long *)malloc(sizeof(long) * NV * size);
    }
    MPI_Gather(row, NV, MPI_LONG, all, NV, MPI_LONG, 0, MPI_COMM_WORLD);
    MPI_Barrier(MPI_COMM_WORLD);
    remove(name);
    if (rank == 0) {
        int q, k;
        for (q = 0; q < size; q++) {
            printf("rank %d:", q);
            for (k = 0; k < NV; k++)
                printf(" %ld", all[q * NV + k]);
            printf("\n");
        }
        free(all);
    }
    MPI_Finalize();
    return 0;
}
