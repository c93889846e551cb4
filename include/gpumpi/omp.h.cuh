#pragma once
#include "gpumpi_prelude.cuh"
#define omp_get_max_threads __gpu_omp_get_max_threads
#define omp_get_num_threads __gpu_omp_get_num_threads
#define omp_get_thread_num __gpu_omp_get_thread_num
#define omp_get_wtime __gpu_omp_get_wtime
