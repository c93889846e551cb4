#ifndef GPUMPI_DATATYPES_CUH
#define GPUMPI_DATATYPES_CUH

#include <stdint.h>
#include <stddef.h>

// Element types used by the pair and complex datatypes.  They are plain
// structs so that device code needs no <complex.h>.
struct gpumpi_cfloat { float re, im; };
struct gpumpi_cdouble { double re, im; };
struct gpumpi_2int { int val; int idx; };
struct gpumpi_float_int { float val; int idx; };
struct gpumpi_double_int { double val; int idx; };
struct gpumpi_long_int { long val; int idx; };

#include "mpi_types_list.cuh"

// MPI_Datatype is an enum, as in gpu_libs/gpu_mpi/datatypes.cuh:12-14, so that
// converted programs may switch over it.  Values >= GPUMPI_FIRST_DERIVED_TYPE
// name contiguous derived types made by MPI_Type_contiguous.
#define GPUMPI_TYPES_ENUM_F(name, type) name
#define GPUMPI_TYPES_ENUM_SEP ,
enum MPI_Datatype {
    GPUMPI_TYPES_LIST(GPUMPI_TYPES_ENUM_F, GPUMPI_TYPES_ENUM_SEP),
    GPUMPI_NUM_BASIC_TYPES,
    MPI_DATATYPE_NULL = 0x7fff,
    GPUMPI_FIRST_DERIVED_TYPE = 0x8000
};
#undef GPUMPI_TYPES_ENUM_F
#undef GPUMPI_TYPES_ENUM_SEP

#endif
