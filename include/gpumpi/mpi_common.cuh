#ifndef GPUMPI_MPI_COMMON_CUH
#define GPUMPI_MPI_COMMON_CUH

// Return codes.  MPI_SUCCESS/MPI_FAILURE/MPI_ERR_OTHER/MPI_UNDEFINED keep the
// values converted programs see (gpu_libs/gpu_mpi/mpi_common.cuh:4-9); the
// remaining codes are this runtime's, returned instead of trapping.
#define MPI_SUCCESS 0
#define MPI_FAILURE -1
#define MPI_ERR_OTHER 1
#define MPI_ERR_BUFFER 2
#define MPI_ERR_COUNT 3
#define MPI_ERR_TYPE 4
#define MPI_ERR_TAG 5
#define MPI_ERR_COMM 6
#define MPI_ERR_RANK 7
#define MPI_ERR_REQUEST 8
#define MPI_ERR_ROOT 9
#define MPI_ERR_OP 10
#define MPI_ERR_ARG 11
#define MPI_ERR_TRUNCATE 12
#define MPI_ERR_INTERN 13
#define MPI_ERR_NO_MEM 14
#define GPUMPI_ERR_TIMEOUT 50      // a bounded device wait ran out
#define GPUMPI_ERR_ABORTED 51      // another rank of the job failed or aborted
#define GPUMPI_ERR_UNSUPPORTED 52  // call exists but this form is not implemented

#define MPI_UNDEFINED -1

#endif
