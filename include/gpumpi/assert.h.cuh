#pragma once
#include "gpumpi_prelude.cuh"
#undef assert
#define assert __gpu_assert
