#pragma once
#include "global_vars.cuh"
#include "mpi.h"

/* Allocator-version spellings the source converter emits
 * (gpu_libs/gpu_mpi/mpi.h.cuh:6-33, mpi.cuh:72-95): on the host they are the
 * plain calls and the coalescing flag is ignored. */
#ifdef __cplusplus
#define HOSTMPI_ATA_VARIANT(suffix)                                                                     \
    static inline int MPI_Alltoall_##suffix(const void* sb, int sc, MPI_Datatype st, void* rb, int rc,  \
                                            MPI_Datatype rt, MPI_Comm comm, bool coalesced = false) {   \
        (void)coalesced;                                                                                \
        return MPI_Alltoall(sb, sc, st, rb, rc, rt, comm);                                              \
    }                                                                                                   \
    static inline int MPI_Alltoallv_##suffix(const void* sb, const int scs[], const int sds[],          \
                                             MPI_Datatype st, void* rb, const int rcs[],                \
                                             const int rds[], MPI_Datatype rt, MPI_Comm comm,           \
                                             bool coalesced = false) {                                  \
        (void)coalesced;                                                                                \
        return MPI_Alltoallv(sb, scs, sds, st, rb, rcs, rds, rt, comm);                                 \
    }
HOSTMPI_ATA_VARIANT(coalesce)
HOSTMPI_ATA_VARIANT(v1)
HOSTMPI_ATA_VARIANT(v2)
HOSTMPI_ATA_VARIANT(v3)
HOSTMPI_ATA_VARIANT(v4)
HOSTMPI_ATA_VARIANT(v5)
HOSTMPI_ATA_VARIANT(v6)
#undef HOSTMPI_ATA_VARIANT

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
#endif
