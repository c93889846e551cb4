#pragma once
#include "gpumpi_prelude.cuh"
