#pragma once
#include "global_vars.cuh"
#include "mpi.h"
