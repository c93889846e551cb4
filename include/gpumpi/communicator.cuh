#ifndef GPUMPI_COMMUNICATOR_CUH
#define GPUMPI_COMMUNICATOR_CUH

#include "group.cuh"

// Opaque communicator handle (gpu_libs/gpu_mpi/communicator.cuh:6-11).
// MPI_COMM_WORLD and MPI_COMM_SELF are sentinel objects: every rank resolves
// them to its own job, so several jobs can share one launch.
struct MPI_Comm_impl;
typedef MPI_Comm_impl* MPI_Comm;

__device__ extern MPI_Comm MPI_COMM_WORLD;
__device__ extern MPI_Comm MPI_COMM_SELF;
__device__ extern MPI_Comm MPI_COMM_NULL;

__device__ int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
__device__ int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm);
__device__ int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm);
__device__ int MPI_Comm_size(MPI_Comm comm, int* size);
__device__ int MPI_Comm_rank(MPI_Comm comm, int* rank);
__device__ int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm);
__device__ int MPI_Comm_free(MPI_Comm* comm);
__device__ int MPI_Comm_compare(MPI_Comm comm1, MPI_Comm comm2, int* result);

__device__ int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[],
                               const int periods[], int reorder, MPI_Comm* comm_cart);
__device__ int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm* comm_new);
__device__ int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]);
__device__ int MPI_Cart_rank(MPI_Comm comm, const int coords[], int* rank);
__device__ int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* rank_source, int* rank_dest);
__device__ int MPI_Dims_create(int nnodes, int ndims, int dims[]);

__device__ int MPI_Attr_get(MPI_Comm comm, int keyval, void* attribute_val, int* flag);
__device__ int MPI_Attr_put(MPI_Comm comm, int keyval, void* attribute_val);

#endif
