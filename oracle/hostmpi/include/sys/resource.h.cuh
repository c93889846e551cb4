#pragma once
#include "../global_vars.cuh"
#include <sys/resource.h>
