#pragma once
#include "global_vars.cuh"
#include <complex.h>
