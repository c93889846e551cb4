#pragma once
#include "gpumpi_prelude.cuh"
#define gethostname __gpu_gethostname
#define getpagesize __gpu_getpagesize
#define sleep __gpu_sleep
#define usleep __gpu_usleep
#define getopt __gpu_getopt
#define optarg (*__gpu_optarg_location())
#define optind (*__gpu_optind_location())
#define opterr (*__gpu_opterr_location())
#define optopt (*__gpu_optopt_location())
