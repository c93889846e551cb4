#pragma once
#include "global_vars.cuh"
#include <limits.h>
