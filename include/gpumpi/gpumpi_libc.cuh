#ifndef GPUMPI_LIBC_CUH
#define GPUMPI_LIBC_CUH

// Device libc subset used by converted programs.  The `*.h.cuh` shim headers
// map the standard names onto these `__gpu_*` functions, with the same names
// the reference shim uses (gpu_libs/gpu_libc/{stdio,stdlib,string,ctype,
// unistd,errno}.h.cuh).  Output is formatted on the device by this runtime's
// own formatter and appended to the job's output buffer, which the launcher
// prints on the host.

#include <stddef.h>
#include <stdint.h>
#include <stdarg.h>
#include <limits.h>
#include <time.h>

typedef struct gpumpi_file_impl __gpu_FILE;
__device__ extern __gpu_FILE* __gpu_stdout;
__device__ extern __gpu_FILE* __gpu_stderr;
__device__ extern __gpu_FILE* __gpu_stdin;

#define __gpu_RAND_MAX 2147483647
#define __gpu_EOF (-1)

// stdio
__device__ int __gpu_printf(const char* format, ...);
__device__ int __gpu_vprintf(const char* format, va_list ap);
__device__ int __gpu_fprintf(__gpu_FILE* stream, const char* format, ...);
__device__ int __gpu_vfprintf(__gpu_FILE* stream, const char* format, va_list ap);
__device__ int __gpu_sprintf(char* str, const char* format, ...);
__device__ int __gpu_snprintf(char* str, size_t size, const char* format, ...);
__device__ int __gpu_vsprintf(char* str, const char* format, va_list ap);
__device__ int __gpu_vsnprintf(char* str, size_t size, const char* format, va_list ap);
__device__ int __gpu_puts(const char* s);
__device__ int __gpu_fputs(const char* s, __gpu_FILE* stream);
__device__ int __gpu_putchar(int c);
__device__ int __gpu_fputc(int c, __gpu_FILE* stream);
__device__ int __gpu_fflush(__gpu_FILE* stream);
__device__ __gpu_FILE* __gpu_fopen(const char* pathname, const char* mode);
__device__ int __gpu_fclose(__gpu_FILE* stream);
__device__ char* __gpu_fgets(char* s, int size, __gpu_FILE* stream);
__device__ int __gpu_fgetc(__gpu_FILE* stream);
__device__ int __gpu_feof(__gpu_FILE* stream);
__device__ int __gpu_fscanf(__gpu_FILE* stream, const char* format, ...);
__device__ size_t __gpu_fwrite(const void* ptr, size_t size, size_t nmemb, __gpu_FILE* stream);
__device__ size_t __gpu_fread(void* ptr, size_t size, size_t nmemb, __gpu_FILE* stream);
__device__ int __gpu_fseek(__gpu_FILE* stream, long offset, int whence);
__device__ long __gpu_ftell(__gpu_FILE* stream);
__device__ void __gpu_rewind(__gpu_FILE* stream);
__device__ int __gpu_remove(const char* pathname);

// stdlib
__device__ void* __gpu_malloc(size_t size);
__device__ void* __gpu_calloc(size_t nmemb, size_t size);
__device__ void* __gpu_realloc(void* ptr, size_t size);
__device__ void __gpu_free(void* ptr);
__device__ int __gpu_posix_memalign(void** memptr, size_t alignment, size_t size);
__device__ void* __gpu_aligned_alloc(size_t alignment, size_t size);
__device__ void __gpu_init_malloc();
__device__ void __gpu_clean_malloc();
__device__ void __gpu_qsort(void* base, size_t nmemb, size_t size,
                            int (*compar)(const void*, const void*));
__device__ void* __gpu_bsearch(const void* key, const void* base, size_t nmemb, size_t size,
                               int (*compar)(const void*, const void*));
__device__ int __gpu_atoi(const char* nptr);
__device__ long __gpu_atol(const char* nptr);
__device__ long long __gpu_atoll(const char* nptr);
__device__ double __gpu_atof(const char* nptr);
__device__ long __gpu_strtol(const char* nptr, char** endptr, int base);
__device__ unsigned long __gpu_strtoul(const char* nptr, char** endptr, int base);
__device__ long long __gpu_strtoll(const char* nptr, char** endptr, int base);
__device__ unsigned long long __gpu_strtoull(const char* nptr, char** endptr, int base);
__device__ double __gpu_strtod(const char* nptr, char** endptr);
__device__ float __gpu_strtof(const char* nptr, char** endptr);
__device__ int __gpu_rand(void);
__device__ void __gpu_srand(unsigned int seed);
__device__ char* __gpu_getenv(const char* name);
__device__ void __gpu_exit(int status);
__device__ void __gpu_abort(void);
__device__ int __gpu_abs(int x);
__device__ long __gpu_labs(long x);

// string
__device__ void* __gpu_memcpy(void* dst, const void* src, size_t n);
__device__ void* __gpu_memmove(void* dst, const void* src, size_t n);
__device__ void* __gpu_memset(void* s, int c, size_t n);
__device__ int __gpu_memcmp(const void* a, const void* b, size_t n);
__device__ void* __gpu_memchr(const void* s, int c, size_t n);
__device__ void* __gpu_memccpy(void* dst, const void* src, int c, size_t n);
__device__ size_t __gpu_strlen(const char* s);
__device__ size_t __gpu_strnlen(const char* s, size_t n);
__device__ char* __gpu_strcpy(char* dst, const char* src);
__device__ char* __gpu_strncpy(char* dst, const char* src, size_t n);
__device__ char* __gpu_strcat(char* dst, const char* src);
__device__ char* __gpu_strncat(char* dst, const char* src, size_t n);
__device__ int __gpu_strcmp(const char* a, const char* b);
__device__ int __gpu_strncmp(const char* a, const char* b, size_t n);
__device__ int __gpu_strcoll(const char* a, const char* b);
__device__ size_t __gpu_strxfrm(char* dst, const char* src, size_t n);
__device__ char* __gpu_strchr(const char* s, int c);
__device__ char* __gpu_strrchr(const char* s, int c);
__device__ size_t __gpu_strspn(const char* s, const char* accept);
__device__ size_t __gpu_strcspn(const char* s, const char* reject);
__device__ char* __gpu_strpbrk(const char* s, const char* accept);
__device__ char* __gpu_strstr(const char* haystack, const char* needle);
__device__ char* __gpu_strtok(char* str, const char* delim);
__device__ char* __gpu_strtok_r(char* str, const char* delim, char** saveptr);
__device__ char* __gpu_strdup(const char* s);
__device__ char* __gpu_strerror(int errnum);

// ctype
__device__ int __gpu_isalnum(int c);
__device__ int __gpu_isalpha(int c);
__device__ int __gpu_islower(int c);
__device__ int __gpu_isupper(int c);
__device__ int __gpu_isdigit(int c);
__device__ int __gpu_isxdigit(int c);
__device__ int __gpu_iscntrl(int c);
__device__ int __gpu_isgraph(int c);
__device__ int __gpu_isspace(int c);
__device__ int __gpu_isblank(int c);
__device__ int __gpu_isprint(int c);
__device__ int __gpu_ispunct(int c);
__device__ int __gpu_tolower(int c);
__device__ int __gpu_toupper(int c);

// errno is per rank
__device__ int* __gpu_errno_location(void);

// unistd / time / omp
__device__ int __gpu_gethostname(char* name, size_t len);
__device__ int __gpu_getpagesize(void);
__device__ unsigned int __gpu_sleep(unsigned int seconds);
__device__ int __gpu_usleep(unsigned int usec);
__device__ int __gpu_getopt(int argc, char* const argv[], const char* optstring);
__device__ char** __gpu_optarg_location(void);
__device__ int* __gpu_optind_location(void);
__device__ int* __gpu_opterr_location(void);
__device__ int* __gpu_optopt_location(void);
struct timeval;
struct timezone;
__device__ int __gpu_gettimeofday(struct timeval* tv, void* tz);
__device__ time_t __gpu_time(time_t* tloc);
__device__ clock_t __gpu_clock(void);
// Parallel loop over the calling rank's thread block (an extension: the
// reference ran one thread per rank).  body(i, arg) runs once for every i in
// [0, n), spread over the block's threads in unspecified order; the call
// returns when all iterations are done.  arg must point to heap or global
// memory (not to the caller's local variables), and the body must not call
// MPI.  Host builds of the same program run the loop in order.
typedef void (*__gpu_loop_body)(long i, void* arg);
__device__ void __gpu_parallel_for(long n, __gpu_loop_body body, void* arg);
__device__ int __gpu_omp_get_max_threads(void);
__device__ int __gpu_omp_get_num_threads(void);
__device__ int __gpu_omp_get_thread_num(void);
// Inside a parallel loop body: the index of the thread block running it within
// the rank (0 unless the job runs each rank as a cluster of blocks).
__device__ int __gpu_loop_block(void);
__device__ double __gpu_omp_get_wtime(void);

// assert: records the failure for the job and ends the rank
__device__ void __gpu_assert_fail(const char* expr, const char* file, int line);
#define __gpu_assert(e) ((e) ? (void)0 : __gpu_assert_fail(#e, __FILE__, __LINE__))

#endif
