#pragma once

// Converted programs include this file in place of <mpi.h>.
#include "mpi.cuh"

// Allocator-version call spellings emitted by the source converter
// (gpu_libs/gpu_mpi/mpi.h.cuh:6-33).  All of them map to the same
// implementation in this runtime.
#if defined(GPUMPI_MALLOC_V1)
#define MPI_Alltoall MPI_Alltoall_v1
#define MPI_Alltoallv MPI_Alltoallv_v1
#elif defined(GPUMPI_MALLOC_V2)
#define MPI_Alltoall MPI_Alltoall_v2
#define MPI_Alltoallv MPI_Alltoallv_v2
#elif defined(GPUMPI_MALLOC_V3)
#define MPI_Alltoall MPI_Alltoall_v3
#define MPI_Alltoallv MPI_Alltoallv_v3
#elif defined(GPUMPI_MALLOC_V4)
#define MPI_Alltoall MPI_Alltoall_v4
#define MPI_Alltoallv MPI_Alltoallv_v4
#elif defined(GPUMPI_MALLOC_V5)
#define MPI_Alltoall MPI_Alltoall_v5
#define MPI_Alltoallv MPI_Alltoallv_v5
#elif defined(GPUMPI_MALLOC_V6)
#define MPI_Alltoall MPI_Alltoall_coalesce
#define MPI_Alltoallv MPI_Alltoallv_coalesce
#elif defined(GPUMPI_MALLOC_V7)
#define MPI_Alltoall MPI_Alltoall_v6
#define MPI_Alltoallv MPI_Alltoallv_v6
#endif
