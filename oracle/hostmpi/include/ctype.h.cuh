#pragma once
#include "global_vars.cuh"
#include <ctype.h>
