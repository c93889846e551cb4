#ifndef GPUMPI_GROUP_CUH
#define GPUMPI_GROUP_CUH

// Opaque group handle (gpu_libs/gpu_mpi/group.cuh:4-9).  WORLD and EMPTY are
// sentinel objects that resolve to the calling rank's job.
struct MPI_Group_impl;
typedef MPI_Group_impl* MPI_Group;

__device__ extern MPI_Group MPI_GROUP_WORLD;
__device__ extern MPI_Group MPI_GROUP_NULL;
__device__ extern MPI_Group MPI_GROUP_EMPTY;

#define MPI_IDENT 0
#define MPI_CONGRUENT 1
#define MPI_SIMILAR 2
#define MPI_UNEQUAL 3

__device__ int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup);
__device__ int MPI_Group_excl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup);
__device__ int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3], MPI_Group* newgroup);
__device__ int MPI_Group_free(MPI_Group* group);
__device__ int MPI_Group_size(MPI_Group group, int* size);
__device__ int MPI_Group_rank(MPI_Group group, int* rank);
__device__ int MPI_Group_translate_ranks(MPI_Group group1, int n, const int ranks1[],
                                         MPI_Group group2, int ranks2[]);

#endif
