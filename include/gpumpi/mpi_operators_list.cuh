// X-macro list of the predefined reduction operators: (handle name, index).
// Same twelve operators, same order as gpu_libs/gpu_mpi/mpi_operators_list.cuh:4-16.
// No include guard: re-expanded where needed.

#define GPUMPI_OPS_LIST(F, SEP) \
    F(MPI_MAX, 0) SEP \
    F(MPI_MIN, 1) SEP \
    F(MPI_SUM, 2) SEP \
    F(MPI_PROD, 3) SEP \
    F(MPI_LAND, 4) SEP \
    F(MPI_BAND, 5) SEP \
    F(MPI_LOR, 6) SEP \
    F(MPI_BOR, 7) SEP \
    F(MPI_LXOR, 8) SEP \
    F(MPI_BXOR, 9) SEP \
    F(MPI_MAXLOC, 10) SEP \
    F(MPI_MINLOC, 11)

#define GPUMPI_NUM_BUILTIN_OPS 12
