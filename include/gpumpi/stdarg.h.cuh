#pragma once
#include "gpumpi_prelude.cuh"
#define vfprintf __gpu_vfprintf
#define vprintf __gpu_vprintf
#define vsprintf __gpu_vsprintf
#define vsnprintf __gpu_vsnprintf
