#pragma once
#include "global_vars.cuh"
#include <stdio.h>
