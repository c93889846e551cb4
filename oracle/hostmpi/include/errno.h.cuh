#pragma once
#include "global_vars.cuh"
#include <errno.h>
