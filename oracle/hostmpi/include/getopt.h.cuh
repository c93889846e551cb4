#pragma once
#include "global_vars.cuh"
#include <getopt.h>
