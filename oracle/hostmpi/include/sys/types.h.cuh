#pragma once
#include "../global_vars.cuh"
#include <sys/types.h>
