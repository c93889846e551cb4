#pragma once
#include "global_vars.cuh"
#include <stdbool.h>
