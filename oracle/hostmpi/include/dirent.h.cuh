#pragma once
#include "global_vars.cuh"
#include <dirent.h>
