#pragma once
#include "global_vars.cuh"
#include <assert.h>
