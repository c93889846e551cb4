#pragma once
#include "gpumpi_prelude.cuh"
#define time __gpu_time
#define clock __gpu_clock
