#pragma once
#include "gpumpi_prelude.cuh"
#undef errno
#define errno (*__gpu_errno_location())
