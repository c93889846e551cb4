#pragma once
#include "global_vars.cuh"
#include <stddef.h>
