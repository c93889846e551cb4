#pragma once
#include "global_vars.cuh"
#include <signal.h>
