#pragma once
#include "../global_vars.cuh"
#include <sys/stat.h>
