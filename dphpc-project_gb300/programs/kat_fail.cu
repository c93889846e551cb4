// Failure scenarios (converter-output form): one rank fails, the others must
// leave their waits with an error code instead of waiting forever.
//   recv_timeout  rank 0 receives a message nobody sends (run with a short
//                 --timeout-ms); the other ranks wait in MPI_Barrier, which
//                 they enter 200 ms later so that rank 0's wait runs out first
//   exit_rank     rank 1 calls exit(3); the others wait in MPI_Barrier
//   abort_rank    rank 2 calls MPI_Abort(5); the others wait in MPI_Recv(ANY)
//   assert_rank   rank 0 fails an assert; the others wait in MPI_Barrier
//   ok            every rank passes the barrier (control)
// Each surviving rank prints the code its call returned.  The reference has no
// counterpart: its waits are unbounded and its errors trap the whole grid
// (gpu_libs/gpu_libc/stdlib.cu:55-63, common/common.h:24-28).
// Usage: kat_fail <scenario> ---gpumpi -n P   (P >= 3)
#include "global_vars.cuh"
#include "mpi.h.cuh"
#include "stdio.h.cuh"
#include "stdlib.h.cuh"
#include "string.h.cuh"
#include "assert.h.cuh"
#include "unistd.h.cuh"

__device__ int __gpu_main(int argc, char** argv) {
    int rank, size, rc = 0, buf = 0;
    MPI_Init(&argc, &argv);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    MPI_Comm_size(MPI_COMM_WORLD, &size);
    const char* sc = argc > 1 ? argv[1] : "ok";
    if (strcmp(sc, "recv_timeout") == 0) {
        if (rank == 0) {
            rc = MPI_Recv(&buf, 1, MPI_INT, 1, 99, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
            printf("rank %d recv rc %d\n", rank, rc);
        } else {
            usleep(200000);
            rc = MPI_Barrier(MPI_COMM_WORLD);
            printf("rank %d barrier rc %d\n", rank, rc);
        }
    } else if (strcmp(sc, "exit_rank") == 0) {
        if (rank == 1) exit(3);
        rc = MPI_Barrier(MPI_COMM_WORLD);
        printf("rank %d barrier rc %d\n", rank, rc);
    } else if (strcmp(sc, "abort_rank") == 0) {
        if (rank == 2) MPI_Abort(MPI_COMM_WORLD, 5);
        rc = MPI_Recv(&buf, 1, MPI_INT, MPI_ANY_SOURCE, 1, MPI_COMM_WORLD, MPI_STATUS_IGNORE);
        printf("rank %d recv rc %d\n", rank, rc);
    } else if (strcmp(sc, "assert_rank") == 0) {
        if (rank == 0) assert(size < 0);
        rc = MPI_Barrier(MPI_COMM_WORLD);
        printf("rank %d barrier rc %d\n", rank, rc);
    } else {
        rc = MPI_Barrier(MPI_COMM_WORLD);
        printf("rank %d barrier rc %d\n", rank, rc);
    }
    MPI_Finalize();
    return rc == MPI_SUCCESS ? 0 : 1;
}

__device__ int __gpu_max_threads() { return 1024; }
