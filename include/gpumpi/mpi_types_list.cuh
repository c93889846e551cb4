// X-macro list of the predefined MPI datatypes: (enum name, C type).
//
// The names, their order and their C types match the datatype enum that
// converted programs are compiled against (gpu_libs/gpu_mpi/mpi_types_list.cuh:3-33),
// so `MPI_Datatype` values are interchangeable.  Entries after MPI_BYTE are
// additions of this runtime (pair types for MAXLOC/MINLOC).
// No include guard: the list macro is re-defined wherever it is expanded.

#define GPUMPI_TYPES_LIST(F, SEP) \
    F(MPI_CHAR, char) SEP \
    F(MPI_SHORT, signed short int) SEP \
    F(MPI_INT, signed int) SEP \
    F(MPI_LONG, signed long int) SEP \
    F(MPI_LONG_LONG_INT, signed long long int) SEP \
    F(MPI_LONG_LONG, signed long long int) SEP \
    F(MPI_SIGNED_CHAR, signed char) SEP \
    F(MPI_UNSIGNED_CHAR, unsigned char) SEP \
    F(MPI_UNSIGNED_SHORT, unsigned short int) SEP \
    F(MPI_UNSIGNED, unsigned int) SEP \
    F(MPI_UNSIGNED_LONG, unsigned long int) SEP \
    F(MPI_UNSIGNED_LONG_LONG, unsigned long long int) SEP \
    F(MPI_FLOAT, float) SEP \
    F(MPI_DOUBLE, double) SEP \
    F(MPI_LONG_DOUBLE, double) SEP \
    F(MPI_WCHAR, wchar_t) SEP \
    F(MPI_C_BOOL, bool) SEP \
    F(MPI_INT8_T, int8_t) SEP \
    F(MPI_INT16_T, int16_t) SEP \
    F(MPI_INT32_T, int32_t) SEP \
    F(MPI_INT64_T, int64_t) SEP \
    F(MPI_UINT8_T, uint8_t) SEP \
    F(MPI_UINT16_T, uint16_t) SEP \
    F(MPI_UINT32_T, uint32_t) SEP \
    F(MPI_UINT64_T, uint64_t) SEP \
    F(MPI_C_COMPLEX, gpumpi_cfloat) SEP \
    F(MPI_C_FLOAT_COMPLEX, gpumpi_cfloat) SEP \
    F(MPI_C_DOUBLE_COMPLEX, gpumpi_cdouble) SEP \
    F(MPI_C_LONG_DOUBLE_COMPLEX, gpumpi_cdouble) SEP \
    F(MPI_BYTE, char) SEP \
    F(MPI_2INT, gpumpi_2int) SEP \
    F(MPI_FLOAT_INT, gpumpi_float_int) SEP \
    F(MPI_DOUBLE_INT, gpumpi_double_int) SEP \
    F(MPI_LONG_INT, gpumpi_long_int) SEP \
    F(MPI_PACKED, char)
