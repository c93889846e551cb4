#pragma once
// <stdio.h> for converted programs (names as in gpu_libs/gpu_libc/stdio.h.cuh).
#include "gpumpi_prelude.cuh"
#undef FILE
#define FILE __gpu_FILE
#undef stdout
#define stdout __gpu_stdout
#undef stderr
#define stderr __gpu_stderr
#undef stdin
#define stdin __gpu_stdin
#undef EOF
#define EOF __gpu_EOF
#define printf __gpu_printf
#define vprintf __gpu_vprintf
#define fprintf __gpu_fprintf
#define sprintf __gpu_sprintf
#define snprintf __gpu_snprintf
#define vsprintf __gpu_vsprintf
#define vsnprintf __gpu_vsnprintf
#define fscanf __gpu_fscanf
#define fflush __gpu_fflush
#define fopen __gpu_fopen
#define fclose __gpu_fclose
#define fgets __gpu_fgets
#define fgetc __gpu_fgetc
#define getc __gpu_fgetc
#define feof __gpu_feof
#define fputs __gpu_fputs
#define fputc __gpu_fputc
#define putc __gpu_fputc
#define putchar __gpu_putchar
#define puts __gpu_puts
#define fwrite __gpu_fwrite
#define fread __gpu_fread
#define fseek __gpu_fseek
#define ftell __gpu_ftell
#define rewind __gpu_rewind
#define remove __gpu_remove
#ifndef SEEK_SET
#define SEEK_SET 0
#define SEEK_CUR 1
#define SEEK_END 2
#endif
