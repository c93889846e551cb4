#pragma once
#include "global_vars.cuh"
#include <float.h>
