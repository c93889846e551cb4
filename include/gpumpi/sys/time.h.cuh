#pragma once
#include "../gpumpi_prelude.cuh"
#define gettimeofday __gpu_gettimeofday
#define time __gpu_time
