#pragma once
#include "global_vars.cuh"
#include <string.h>
