#pragma once
#include "global_vars.cuh"
#include <math.h>
