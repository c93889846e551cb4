#pragma once
#include "global_vars.cuh"
#include <inttypes.h>
