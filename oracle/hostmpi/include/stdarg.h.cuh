#pragma once
#include "global_vars.cuh"
#include <stdarg.h>
