#pragma once
#include "global_vars.cuh"
#include <stdint.h>
