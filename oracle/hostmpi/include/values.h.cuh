#pragma once
#include "global_vars.cuh"
