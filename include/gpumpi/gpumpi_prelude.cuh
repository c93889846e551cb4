#ifndef GPUMPI_PRELUDE_CUH
#define GPUMPI_PRELUDE_CUH
// Every libc header a converted program may name is pulled in once, before
// any shim macro exists, so the order of the program's includes never matters.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#include <math.h>
#include <float.h>
#include <stdarg.h>
#include <stdint.h>
#include <inttypes.h>
#include <limits.h>
#include <errno.h>
#include <time.h>
#include <signal.h>
#include <assert.h>
#include <stddef.h>
#include <stdbool.h>
#include <unistd.h>
#include <getopt.h>
#include <sys/time.h>
#include <sys/types.h>
#include <sys/stat.h>
#include <sys/resource.h>
#include <dirent.h>
#include "gpumpi_libc.cuh"
#endif
