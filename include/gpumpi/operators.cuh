#ifndef GPUMPI_OPERATORS_CUH
#define GPUMPI_OPERATORS_CUH

#include "datatypes.cuh"
#include "mpi_operators_list.cuh"

// Opaque reduction-operator handle (gpu_libs/gpu_mpi/operators.cuh:7-20).
struct MPI_Op_impl;
typedef MPI_Op_impl* MPI_Op;

#define GPUMPI_OP_DECL_F(name, idx) __device__ extern MPI_Op name;
#define GPUMPI_OP_DECL_SEP
GPUMPI_OPS_LIST(GPUMPI_OP_DECL_F, GPUMPI_OP_DECL_SEP)
#undef GPUMPI_OP_DECL_F
#undef GPUMPI_OP_DECL_SEP

// inoutvec[i] = invec[i] (op) inoutvec[i] for i < *len.
typedef void MPI_User_function(void* invec, void* inoutvec, int* len, MPI_Datatype* datatype);

#define MPI_OP_NULL ((MPI_Op)0)

__device__ int MPI_Op_create(MPI_User_function* user_fn, int commute, MPI_Op* op);
__device__ int MPI_Op_free(MPI_Op* op);

#endif
