#pragma once
/* Host build of converter-form programs: one process per rank, so the
 * per-rank global arrays need only one element and device qualifiers vanish.
 * TEST INFRASTRUCTURE ONLY (hostmpi oracle). */
#ifndef __device__
#define __device__
#endif
#ifndef __host__
#define __host__
#endif
#define __gpu_global(var) (var[0])
#define __gpu_main hostmpi_user_main
#ifndef GPU_MPI_MAX_RANKS
#define GPU_MPI_MAX_RANKS 1024
#endif
#ifdef __cplusplus
extern "C" int hostmpi_user_main(int argc, char** argv);
#endif
