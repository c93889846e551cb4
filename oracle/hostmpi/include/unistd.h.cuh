#pragma once
#include "global_vars.cuh"
#include <unistd.h>
