#pragma once
#include "global_vars.cuh"
#include <time.h>
