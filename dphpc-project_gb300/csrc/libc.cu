// Device libc subset for converted programs (the `__gpu_*` functions the shim
// headers map to, as in gpu_libs/gpu_libc/*.h.cuh).  Formatted output goes to
// the job's stdout/stderr buffers through the exact formatter in fmt.h; the
// reference used a vendored tiny printf (gpu_libs/gpu_libc/mp4_printf.cu).
// rand() reproduces the C library's additive-feedback generator (state
// r[i] = r[i-3] + r[i-31], seeded through x -> 16807 x mod (2^31 - 1)), so a
// program draws the same numbers on the GPU as on the host.
#include <stdarg.h>
#include <sys/time.h>

#include "fmt.h"
#include "gpumpi_libc.cuh"
#include "rt.cuh"

using namespace gm;

constexpr int FILE_BUF = HOSTCALL_DATA;

struct gpumpi_file_impl {
    int stream;        // 1 stdout, 2 stderr, 0 stdin, 3 a host file opened through the launcher
    int eof;
    int wlen;          // bytes buffered for writing
    int rpos, rlen;    // unread window of the read buffer
    long long handle;  // the launcher's handle of a host file
    char* wbuf;        // [FILE_BUF] (host files only)
    char* rbuf;        // [FILE_BUF]
};

__device__ gpumpi_file_impl gm_file_stdout = {1, 0, 0, 0, 0, -1, nullptr, nullptr};
__device__ gpumpi_file_impl gm_file_stderr = {2, 0, 0, 0, 0, -1, nullptr, nullptr};
__device__ gpumpi_file_impl gm_file_stdin = {0, 0, 0, 0, 0, -1, nullptr, nullptr};
__device__ __gpu_FILE* __gpu_stdout = &gm_file_stdout;
__device__ __gpu_FILE* __gpu_stderr = &gm_file_stderr;
__device__ __gpu_FILE* __gpu_stdin = &gm_file_stdin;

// ---------------------------------------------------------------- host files
// The rank's leader calls the launcher through its HostCall slot (mapped host
// memory, system-scope release/acquire).  Returns the answer's ret; on failure
// (ret < 0) errno is set.  Without a host service (collective API, serving)
// every call fails with ENOENT, as fopen did before there was one.
static __device__ long long host_call(u32 op, long long a0, long long a1, long long a2, const void* in,
                                      u32 in_len, void* out, u32 out_cap, u32* out_len) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    if (out_len) *out_len = 0;
    if (!j->hcall) {
        b.priv->errno_v = 2;   // ENOENT
        return -1;
    }
    HostCall* h = &j->hcall[b.rank];
    h->op = op;
    h->a[0] = a0;
    h->a[1] = a1;
    h->a[2] = a2;
    h->len = in_len;
    for (u32 i = 0; i < in_len; i++) h->data[i] = ((const char*)in)[i];
    __threadfence_system();
    asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(&h->state), "r"(1u) : "memory");
    const u64 t0 = gtime();
    unsigned ns = 256;
    for (;;) {
        u32 st;
        asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(st) : "l"(&h->state) : "memory");
        if (st == 2) break;
        if (ld_relaxed_int(&j->status[0]) != 0) {
            b.priv->errno_v = 5;   // EIO
            return -1;
        }
        if (gtime() - t0 > j->timeout_ns) {
            job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "host file call timed out");
            b.priv->errno_v = 5;
            return -1;
        }
        __nanosleep(ns);
        if (ns < 8192) ns <<= 1;
    }
    const volatile HostCall* vh = h;
    const long long ret = vh->ret;
    const int err = vh->err;
    u32 n = vh->len;
    if (n > out_cap) n = out_cap;
    for (u32 i = 0; i < n; i++) ((char*)out)[i] = vh->data[i];
    if (out_len) *out_len = n;
    h->state = 0u;   // the next request's release orders this store before its own
    if (ret < 0) b.priv->errno_v = err;
    return ret;
}

static __device__ int file_flush_write(gpumpi_file_impl* f) {
    int rc = 0;
    if (f->wlen > 0) {
        const long long r = host_call(HC_WRITE, f->handle, 0, 0, f->wbuf, (u32)f->wlen, nullptr, 0, nullptr);
        if (r != f->wlen) rc = -1;
        f->wlen = 0;
    }
    return rc;
}

static __device__ int file_write(gpumpi_file_impl* f, const char* p, u64 n) {
    if (f->rpos < f->rlen) {   // writing after reading: drop the unread window, position at it
        host_call(HC_SEEK, f->handle, -(long long)(f->rlen - f->rpos), 1, nullptr, 0, nullptr, 0, nullptr);
        f->rpos = f->rlen = 0;
    }
    u64 done = 0;
    while (done < n) {
        u64 k = (u64)(FILE_BUF - f->wlen);
        if (k > n - done) k = n - done;
        for (u64 i = 0; i < k; i++) f->wbuf[f->wlen + i] = p[done + i];
        f->wlen += (int)k;
        done += k;
        if (f->wlen == FILE_BUF && file_flush_write(f)) return -1;
    }
    return 0;
}

// Refill the read buffer; 0 bytes: end of file (or an error).
static __device__ int file_fill(gpumpi_file_impl* f) {
    if (file_flush_write(f)) return 0;
    u32 got = 0;
    const long long r = host_call(HC_READ, f->handle, FILE_BUF, 0, nullptr, 0, f->rbuf, FILE_BUF, &got);
    f->rpos = 0;
    f->rlen = r > 0 ? (int)got : 0;
    if (f->rlen == 0) f->eof = 1;
    return f->rlen;
}

static __device__ int file_getc(gpumpi_file_impl* f) {
    if (f->rpos == f->rlen && file_fill(f) == 0) return -1;
    return (unsigned char)f->rbuf[f->rpos++];
}

static __device__ bool host_file(const __gpu_FILE* f) { return f && f->stream == 3; }

// ---------------------------------------------------------------- stdio
static __device__ int emit(int stream, const char* fmt, va_list ap) {
    Job* j = bctx().job;
    char line[OUT_LINE_MAX];
    va_list ap2;
    va_copy(ap2, ap);
    int n = gmfmt::vformat(line, sizeof(line), fmt, ap);
    if (n < (int)sizeof(line)) {
        out_write(j, stream, line, n);
    } else {
        char* big = (char*)heap_alloc(&j->heap, (u64)n + 1);
        if (big) {
            gmfmt::vformat(big, (size_t)n + 1, fmt, ap2);
            out_write(j, stream, big, n);
            heap_free(&j->heap, big);
        } else {
            out_write(j, stream, line, (int)sizeof(line) - 1);
        }
    }
    va_end(ap2);
    return n;
}

__device__ int __gpu_vprintf(const char* format, va_list ap) { return emit(1, format, ap); }

__device__ int __gpu_printf(const char* format, ...) {
    va_list ap;
    va_start(ap, format);
    int n = emit(1, format, ap);
    va_end(ap);
    return n;
}

__device__ int __gpu_vfprintf(__gpu_FILE* stream, const char* format, va_list ap) {
    if (!stream || stream->stream == 0) return -1;
    if (host_file(stream)) {
        Job* j = bctx().job;
        char line[OUT_LINE_MAX];
        va_list ap2;
        va_copy(ap2, ap);
        const int n = gmfmt::vformat(line, sizeof(line), format, ap);
        int rc;
        if (n < (int)sizeof(line)) {
            rc = file_write(stream, line, (u64)n);
        } else {
            char* big = (char*)heap_alloc(&j->heap, (u64)n + 1);
            if (!big) {
                va_end(ap2);
                return -1;
            }
            gmfmt::vformat(big, (size_t)n + 1, format, ap2);
            rc = file_write(stream, big, (u64)n);
            heap_free(&j->heap, big);
        }
        va_end(ap2);
        return rc ? -1 : n;
    }
    return emit(stream->stream, format, ap);
}

__device__ int __gpu_fprintf(__gpu_FILE* stream, const char* format, ...) {
    va_list ap;
    va_start(ap, format);
    int n = __gpu_vfprintf(stream, format, ap);
    va_end(ap);
    return n;
}

__device__ int __gpu_vsnprintf(char* str, size_t size, const char* format, va_list ap) {
    return gmfmt::vformat(str, size, format, ap);
}

__device__ int __gpu_vsprintf(char* str, const char* format, va_list ap) {
    return gmfmt::vformat(str, (size_t)1 << 30, format, ap);
}

__device__ int __gpu_sprintf(char* str, const char* format, ...) {
    va_list ap;
    va_start(ap, format);
    int n = gmfmt::vformat(str, (size_t)1 << 30, format, ap);
    va_end(ap);
    return n;
}

__device__ int __gpu_snprintf(char* str, size_t size, const char* format, ...) {
    va_list ap;
    va_start(ap, format);
    int n = gmfmt::vformat(str, size, format, ap);
    va_end(ap);
    return n;
}

__device__ int __gpu_fputs(const char* s, __gpu_FILE* stream) {
    if (!stream || stream->stream == 0) return -1;
    int n = 0;
    while (s[n]) n++;
    if (host_file(stream)) return file_write(stream, s, (u64)n) ? -1 : n;
    out_write(bctx().job, stream->stream, s, n);
    return n;
}

__device__ int __gpu_puts(const char* s) {
    int n = __gpu_fputs(s, __gpu_stdout);
    out_write(bctx().job, 1, "\n", 1);
    return n + 1;
}

__device__ int __gpu_fputc(int c, __gpu_FILE* stream) {
    if (!stream || stream->stream == 0) return -1;
    char ch = (char)c;
    if (host_file(stream)) return file_write(stream, &ch, 1) ? -1 : (unsigned char)ch;
    out_write(bctx().job, stream->stream, &ch, 1);
    return (unsigned char)ch;
}

__device__ int __gpu_putchar(int c) { return __gpu_fputc(c, __gpu_stdout); }

__device__ size_t __gpu_fwrite(const void* ptr, size_t size, size_t nmemb, __gpu_FILE* stream) {
    if (!stream || stream->stream == 0) return 0;
    if (host_file(stream)) return file_write(stream, (const char*)ptr, (u64)size * nmemb) ? 0 : nmemb;
    out_write(bctx().job, stream->stream, (const char*)ptr, (int)(size * nmemb));
    return nmemb;
}

__device__ int __gpu_fflush(__gpu_FILE* stream) {
    if (!host_file(stream)) return 0;
    if (file_flush_write(stream)) return -1;
    return host_call(HC_FLUSH, stream->handle, 0, 0, nullptr, 0, nullptr, 0, nullptr) < 0 ? -1 : 0;
}

// Files are opened, read and written by the launcher on the rank's behalf
// (host_call); each open file keeps a write buffer and a read buffer of
// HOSTCALL_DATA bytes in the device heap.  The reference's stubs trapped
// (gpu_libs/gpu_libc/stdio.cu:21-76) and its host-side processor was empty
// (gpu_libs/gpu_main/libc_processor.cu:3-5).
__device__ __gpu_FILE* __gpu_fopen(const char* pathname, const char* mode) {
    if (!pathname || !mode) return nullptr;
    char req[512];
    u32 n = 0;
    for (const char* p = pathname; *p; p++) {
        if (n + 2 >= sizeof(req)) {
            bctx().priv->errno_v = 36;   // ENAMETOOLONG
            return nullptr;
        }
        req[n++] = *p;
    }
    req[n++] = 0;
    for (const char* p = mode; *p && n + 1 < sizeof(req); p++) req[n++] = *p;
    req[n++] = 0;
    Job* j = bctx().job;
    gpumpi_file_impl* f = (gpumpi_file_impl*)heap_alloc(&j->heap, sizeof(gpumpi_file_impl) + 2 * FILE_BUF);
    if (!f) {
        bctx().priv->errno_v = 12;   // ENOMEM
        return nullptr;
    }
    const long long h = host_call(HC_OPEN, 0, 0, 0, req, n, nullptr, 0, nullptr);
    if (h < 0) {
        heap_free(&j->heap, f);
        return nullptr;
    }
    f->stream = 3;
    f->eof = 0;
    f->wlen = 0;
    f->rpos = f->rlen = 0;
    f->handle = h;
    f->wbuf = (char*)(f + 1);
    f->rbuf = f->wbuf + FILE_BUF;
    return f;
}

__device__ int __gpu_fclose(__gpu_FILE* stream) {
    if (!stream) return -1;
    if (!host_file(stream)) return 0;
    int rc = file_flush_write(stream);
    if (host_call(HC_CLOSE, stream->handle, 0, 0, nullptr, 0, nullptr, 0, nullptr) < 0) rc = -1;
    heap_free(&bctx().job->heap, stream);
    return rc;
}

__device__ char* __gpu_fgets(char* s, int size, __gpu_FILE* stream) {
    if (!host_file(stream) || size <= 0) return nullptr;
    int n = 0;
    while (n < size - 1) {
        const int c = file_getc(stream);
        if (c < 0) break;
        s[n++] = (char)c;
        if (c == '\n') break;
    }
    if (n == 0) return nullptr;
    s[n] = 0;
    return s;
}

__device__ int __gpu_fgetc(__gpu_FILE* stream) {
    if (!host_file(stream)) return -1;
    return file_getc(stream);
}

__device__ int __gpu_feof(__gpu_FILE* stream) {
    if (!host_file(stream)) return 1;
    return stream->eof && stream->rpos == stream->rlen;
}

__device__ int __gpu_fscanf(__gpu_FILE* stream, const char* format, ...) {
    (void)stream;
    (void)format;
    return -1;
}

__device__ size_t __gpu_fread(void* ptr, size_t size, size_t nmemb, __gpu_FILE* stream) {
    if (!host_file(stream) || size == 0) return 0;
    const u64 want = (u64)size * nmemb;
    char* d = (char*)ptr;
    u64 got = 0;
    while (got < want) {
        if (stream->rpos == stream->rlen && file_fill(stream) == 0) break;
        u64 k = (u64)(stream->rlen - stream->rpos);
        if (k > want - got) k = want - got;
        for (u64 i = 0; i < k; i++) d[got + i] = stream->rbuf[stream->rpos + i];
        stream->rpos += (int)k;
        got += k;
    }
    return got / size;
}

__device__ int __gpu_fseek(__gpu_FILE* stream, long offset, int whence) {
    if (!host_file(stream)) return -1;
    if (file_flush_write(stream)) return -1;
    long long off = offset;
    if (whence == 1) off -= (long long)(stream->rlen - stream->rpos);   // SEEK_CUR: from the user's position
    stream->rpos = stream->rlen = 0;
    stream->eof = 0;
    return host_call(HC_SEEK, stream->handle, off, whence, nullptr, 0, nullptr, 0, nullptr) < 0 ? -1 : 0;
}

__device__ long __gpu_ftell(__gpu_FILE* stream) {
    if (!host_file(stream)) return -1;
    const long long pos = host_call(HC_TELL, stream->handle, 0, 0, nullptr, 0, nullptr, 0, nullptr);
    if (pos < 0) return -1;
    return (long)(pos - (stream->rlen - stream->rpos) + stream->wlen);
}

__device__ void __gpu_rewind(__gpu_FILE* stream) {
    if (__gpu_fseek(stream, 0, 0) == 0) stream->eof = 0;
}

__device__ int __gpu_remove(const char* pathname) {
    u32 n = 0;
    char req[512];
    for (const char* p = pathname; *p; p++) {
        if (n + 1 >= sizeof(req)) return -1;
        req[n++] = *p;
    }
    req[n++] = 0;
    return host_call(HC_REMOVE, 0, 0, 0, req, n, nullptr, 0, nullptr) < 0 ? -1 : 0;
}

// ---------------------------------------------------------------- memory
static __device__ bool can_fan_out(u64 n) {
    BlockCtx& b = bctx();
    return n >= 65536 && b.leader_mode && threadIdx.x == 0 && !b.in_call;
}

__device__ void* __gpu_malloc(size_t size) { return heap_alloc(&bctx().job->heap, size); }

// Parallel loop over the rank's whole thread block (over every block of the
// rank's cluster when the job runs ranks as clusters, see cluster.cu).  The
// leader hands the loop to the block like an MPI call; each thread runs
// iterations tid, tid+T, ... (tid counts the threads of the whole cluster);
// the call returns after a block barrier, so every iteration's writes are
// visible to the leader.  `arg` is passed to every thread, so it must point to
// memory all threads can read (heap, globals); pointers into the leader's
// local memory, nested calls and calls from inside an MPI call run the loop
// on the leader alone, in order.
__device__ void __gpu_parallel_for(long n, __gpu_loop_body body, void* arg) {
    BlockCtx& b = bctx();
    if (n <= 0) return;
    const bool fan = n > 1 && b.leader_mode && threadIdx.x == 0 && !b.in_call && (arg == nullptr || is_global(arg));
    if (!fan) {
        for (long i = 0; i < n; i++) body(i, arg);
        return;
    }
    Call call;
    call.op = OP_PARFOR;
    call.a[0] = (u64)body;
    call.a[1] = (u64)arg;
    call.a[2] = (u64)n;
    block_call(call);
}

__device__ void* __gpu_memset(void* s, int c, size_t n) {
    if (can_fan_out(n) && is_global(s)) {
        Call call;
        call.op = OP_MEMSET;
        call.a[0] = (u64)s;
        call.a[1] = (u64)c;
        call.a[2] = n;
        block_call(call);
        return s;
    }
    unsigned char* d = (unsigned char*)s;
    for (size_t i = 0; i < n; i++) d[i] = (unsigned char)c;
    return s;
}

__device__ void* __gpu_calloc(size_t nmemb, size_t size) {
    size_t n = nmemb * size;
    if (size && n / size != nmemb) return nullptr;
    void* p = heap_alloc(&bctx().job->heap, n);
    if (p) __gpu_memset(p, 0, n);
    return p;
}

__device__ void __gpu_free(void* ptr) { heap_free(&bctx().job->heap, ptr); }

__device__ void* __gpu_memcpy(void* dst, const void* src, size_t n) {
    if (can_fan_out(n) && is_global(dst) && is_global(src)) {
        Call call;
        call.op = OP_MEMCPY;
        call.a[0] = (u64)dst;
        call.a[1] = (u64)src;
        call.a[2] = n;
        block_call(call);
        return dst;
    }
    char* d = (char*)dst;
    const char* s = (const char*)src;
    if ((((uintptr_t)d | (uintptr_t)s | n) & 7) == 0) {
        for (size_t i = 0; i < n / 8; i++) ((u64*)d)[i] = ((const u64*)s)[i];
    } else {
        for (size_t i = 0; i < n; i++) d[i] = s[i];
    }
    return dst;
}

__device__ void* __gpu_memmove(void* dst, const void* src, size_t n) {
    char* d = (char*)dst;
    const char* s = (const char*)src;
    if (d == s || n == 0) return dst;
    if (d < s || d >= s + n) {
        for (size_t i = 0; i < n; i++) d[i] = s[i];
    } else {
        for (size_t i = n; i > 0; i--) d[i - 1] = s[i - 1];
    }
    return dst;
}

__device__ void* __gpu_realloc(void* ptr, size_t size) {
    Heap* h = &bctx().job->heap;
    if (!ptr) return heap_alloc(h, size);
    if (size == 0) {
        heap_free(h, ptr);
        return nullptr;
    }
    u64 old = heap_usable_size(h, ptr);
    if (old >= size) return ptr;
    void* p = heap_alloc(h, size);
    if (!p) return nullptr;
    __gpu_memcpy(p, ptr, old < size ? old : size);
    heap_free(h, ptr);
    return p;
}

__device__ int __gpu_posix_memalign(void** memptr, size_t alignment, size_t size) {
    // Chunks of class c are aligned to min(16 << c, 64 KiB); round the size up.
    if (alignment == 0 || (alignment & (alignment - 1))) return 22;  // EINVAL
    size_t want = size < alignment ? alignment : size;
    void* p = heap_alloc(&bctx().job->heap, want);
    if (!p) return 12;  // ENOMEM
    if (((uintptr_t)p & (alignment - 1)) != 0) {
        heap_free(&bctx().job->heap, p);
        return 12;
    }
    *memptr = p;
    return 0;
}

__device__ void* __gpu_aligned_alloc(size_t alignment, size_t size) {
    void* p = nullptr;
    return __gpu_posix_memalign(&p, alignment, size) == 0 ? p : nullptr;
}

__device__ void __gpu_init_malloc() {}
__device__ void __gpu_clean_malloc() {}

// ---------------------------------------------------------------- exit / assert
__device__ void __gpu_exit(int status) { rank_exit_now(status); }

__device__ void __gpu_abort(void) {
    out_write(bctx().job, 2, "Aborted\n", 8);
    rank_exit_now(134);
}

__device__ void __gpu_assert_fail(const char* expr, const char* file, int line) {
    char buf[512];
    int n = gmfmt::format(buf, sizeof(buf), "GPUMPI rank %d: %s:%d: Assertion `%s' failed.\n",
                          bctx().rank, file, line, expr);
    out_write(bctx().job, 2, buf, n < (int)sizeof(buf) ? n : (int)sizeof(buf) - 1);
    rank_exit_now(134);
}

__device__ int __gpu_abs(int x) { return x < 0 ? -x : x; }
__device__ long __gpu_labs(long x) { return x < 0 ? -x : x; }

// ---------------------------------------------------------------- rand
static __device__ void rnd_seed(RankPriv* p, unsigned int seed) {
    int r[34];
    r[0] = (int)(seed ? seed : 1u);
    for (int i = 1; i < 31; i++) {
        long long v = (16807LL * r[i - 1]) % 2147483647LL;
        if (v < 0) v += 2147483647LL;
        r[i] = (int)v;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 0; i < 34; i++) p->rnd[i] = (unsigned)r[i];
    p->rnd_i = 0;
    // discard the first 310 outputs
    for (int k = 34; k < 344; k++) {
        unsigned v = p->rnd[(p->rnd_i + 34 - 31) % 34] + p->rnd[(p->rnd_i + 34 - 3) % 34];
        p->rnd[p->rnd_i] = v;
        p->rnd_i = (p->rnd_i + 1) % 34;
    }
    p->rnd_seeded = 1;
}

__device__ void __gpu_srand(unsigned int seed) { rnd_seed(bctx().priv, seed); }

__device__ int __gpu_rand(void) {
    RankPriv* p = bctx().priv;
    if (!p->rnd_seeded) rnd_seed(p, 1);
    unsigned v = p->rnd[(p->rnd_i + 34 - 31) % 34] + p->rnd[(p->rnd_i + 34 - 3) % 34];
    p->rnd[p->rnd_i] = v;
    p->rnd_i = (p->rnd_i + 1) % 34;
    return (int)(v >> 1);
}

// ---------------------------------------------------------------- sorting
static __device__ void swap_bytes(char* a, char* b, size_t n) {
    for (size_t i = 0; i < n; i++) {
        char t = a[i];
        a[i] = b[i];
        b[i] = t;
    }
}

// Stable bottom-up merge sort through a heap buffer; insertion sort when the
// buffer cannot be had.
__device__ void __gpu_qsort(void* base, size_t nmemb, size_t size,
                            int (*compar)(const void*, const void*)) {
    if (nmemb < 2 || size == 0) return;
    char* a = (char*)base;
    char* tmp = (char*)heap_alloc(&bctx().job->heap, nmemb * size);
    if (!tmp) {
        for (size_t i = 1; i < nmemb; i++)
            for (size_t k = i; k > 0 && compar(a + (k - 1) * size, a + k * size) > 0; k--)
                swap_bytes(a + (k - 1) * size, a + k * size, size);
        return;
    }
    char* src = a;
    char* dst = tmp;
    for (size_t w = 1; w < nmemb; w *= 2) {
        for (size_t lo = 0; lo < nmemb; lo += 2 * w) {
            size_t mid = lo + w < nmemb ? lo + w : nmemb;
            size_t hi = lo + 2 * w < nmemb ? lo + 2 * w : nmemb;
            size_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) {
                const char* pick;
                if (compar(src + j * size, src + i * size) < 0) pick = src + (j++) * size;
                else pick = src + (i++) * size;
                for (size_t b = 0; b < size; b++) dst[k * size + b] = pick[b];
                k++;
            }
            while (i < mid) {
                for (size_t b = 0; b < size; b++) dst[k * size + b] = src[i * size + b];
                i++;
                k++;
            }
            while (j < hi) {
                for (size_t b = 0; b < size; b++) dst[k * size + b] = src[j * size + b];
                j++;
                k++;
            }
        }
        char* t = src;
        src = dst;
        dst = t;
    }
    if (src != a) __gpu_memcpy(a, src, nmemb * size);
    heap_free(&bctx().job->heap, tmp);
}

__device__ void* __gpu_bsearch(const void* key, const void* base, size_t nmemb, size_t size,
                               int (*compar)(const void*, const void*)) {
    size_t lo = 0, hi = nmemb;
    while (lo < hi) {
        size_t mid = lo + (hi - lo) / 2;
        const char* p = (const char*)base + mid * size;
        int c = compar(key, p);
        if (c == 0) return (void*)p;
        if (c < 0) hi = mid;
        else lo = mid + 1;
    }
    return nullptr;
}

// ---------------------------------------------------------------- ctype
__device__ int __gpu_isdigit(int c) { return c >= '0' && c <= '9'; }
__device__ int __gpu_islower(int c) { return c >= 'a' && c <= 'z'; }
__device__ int __gpu_isupper(int c) { return c >= 'A' && c <= 'Z'; }
__device__ int __gpu_isalpha(int c) { return __gpu_islower(c) || __gpu_isupper(c); }
__device__ int __gpu_isalnum(int c) { return __gpu_isalpha(c) || __gpu_isdigit(c); }
__device__ int __gpu_isxdigit(int c) {
    return __gpu_isdigit(c) || (c >= 'a' && c <= 'f') || (c >= 'A' && c <= 'F');
}
__device__ int __gpu_iscntrl(int c) { return (c >= 0 && c < 32) || c == 127; }
__device__ int __gpu_isgraph(int c) { return c > 32 && c < 127; }
__device__ int __gpu_isprint(int c) { return c >= 32 && c < 127; }
__device__ int __gpu_isspace(int c) { return c == ' ' || (c >= 9 && c <= 13); }
__device__ int __gpu_isblank(int c) { return c == ' ' || c == '\t'; }
__device__ int __gpu_ispunct(int c) { return __gpu_isgraph(c) && !__gpu_isalnum(c); }
__device__ int __gpu_tolower(int c) { return __gpu_isupper(c) ? c + 32 : c; }
__device__ int __gpu_toupper(int c) { return __gpu_islower(c) ? c - 32 : c; }

// ---------------------------------------------------------------- strings
__device__ size_t __gpu_strlen(const char* s) {
    size_t n = 0;
    while (s[n]) n++;
    return n;
}
__device__ size_t __gpu_strnlen(const char* s, size_t m) {
    size_t n = 0;
    while (n < m && s[n]) n++;
    return n;
}
__device__ char* __gpu_strcpy(char* d, const char* s) {
    size_t i = 0;
    while ((d[i] = s[i])) i++;
    return d;
}
__device__ char* __gpu_strncpy(char* d, const char* s, size_t n) {
    size_t i = 0;
    for (; i < n && s[i]; i++) d[i] = s[i];
    for (; i < n; i++) d[i] = 0;
    return d;
}
__device__ char* __gpu_strcat(char* d, const char* s) {
    __gpu_strcpy(d + __gpu_strlen(d), s);
    return d;
}
__device__ char* __gpu_strncat(char* d, const char* s, size_t n) {
    size_t l = __gpu_strlen(d), i = 0;
    for (; i < n && s[i]; i++) d[l + i] = s[i];
    d[l + i] = 0;
    return d;
}
__device__ int __gpu_strcmp(const char* a, const char* b) {
    while (*a && *a == *b) {
        a++;
        b++;
    }
    return (unsigned char)*a - (unsigned char)*b;
}
__device__ int __gpu_strncmp(const char* a, const char* b, size_t n) {
    for (size_t i = 0; i < n; i++) {
        if (a[i] != b[i] || !a[i]) return (unsigned char)a[i] - (unsigned char)b[i];
    }
    return 0;
}
__device__ int __gpu_strcoll(const char* a, const char* b) { return __gpu_strcmp(a, b); }
__device__ size_t __gpu_strxfrm(char* d, const char* s, size_t n) {
    size_t l = __gpu_strlen(s);
    if (n) __gpu_strncpy(d, s, n);
    return l;
}
__device__ char* __gpu_strchr(const char* s, int c) {
    for (;; s++) {
        if (*s == (char)c) return (char*)s;
        if (!*s) return nullptr;
    }
}
__device__ char* __gpu_strrchr(const char* s, int c) {
    const char* r = nullptr;
    for (;; s++) {
        if (*s == (char)c) r = s;
        if (!*s) return (char*)r;
    }
}
__device__ size_t __gpu_strspn(const char* s, const char* acc) {
    size_t n = 0;
    while (s[n] && __gpu_strchr(acc, s[n])) n++;
    return n;
}
__device__ size_t __gpu_strcspn(const char* s, const char* rej) {
    size_t n = 0;
    while (s[n] && !__gpu_strchr(rej, s[n])) n++;
    return n;
}
__device__ char* __gpu_strpbrk(const char* s, const char* acc) {
    s += __gpu_strcspn(s, acc);
    return *s ? (char*)s : nullptr;
}
__device__ char* __gpu_strstr(const char* h, const char* nd) {
    size_t ln = __gpu_strlen(nd);
    if (!ln) return (char*)h;
    for (; *h; h++)
        if (__gpu_strncmp(h, nd, ln) == 0) return (char*)h;
    return nullptr;
}
__device__ char* __gpu_strtok_r(char* str, const char* delim, char** save) {
    char* s = str ? str : *save;
    if (!s) return nullptr;
    s += __gpu_strspn(s, delim);
    if (!*s) {
        *save = nullptr;
        return nullptr;
    }
    char* e = s + __gpu_strcspn(s, delim);
    if (*e) {
        *e = 0;
        *save = e + 1;
    } else {
        *save = nullptr;
    }
    return s;
}
__device__ char* __gpu_strtok(char* str, const char* delim) {
    return __gpu_strtok_r(str, delim, &bctx().priv->strtok_save);
}
__device__ char* __gpu_strdup(const char* s) {
    size_t n = __gpu_strlen(s) + 1;
    char* d = (char*)heap_alloc(&bctx().job->heap, n);
    if (d) __gpu_memcpy(d, s, n);
    return d;
}
__device__ char* __gpu_strerror(int errnum) {
    (void)errnum;
    static __device__ char msg[] = "device error";
    return msg;
}
__device__ int __gpu_memcmp(const void* a, const void* b, size_t n) {
    const unsigned char* x = (const unsigned char*)a;
    const unsigned char* y = (const unsigned char*)b;
    for (size_t i = 0; i < n; i++)
        if (x[i] != y[i]) return x[i] - y[i];
    return 0;
}
__device__ void* __gpu_memchr(const void* s, int c, size_t n) {
    const unsigned char* p = (const unsigned char*)s;
    for (size_t i = 0; i < n; i++)
        if (p[i] == (unsigned char)c) return (void*)(p + i);
    return nullptr;
}
__device__ void* __gpu_memccpy(void* dst, const void* src, int c, size_t n) {
    unsigned char* d = (unsigned char*)dst;
    const unsigned char* s = (const unsigned char*)src;
    for (size_t i = 0; i < n; i++) {
        d[i] = s[i];
        if (s[i] == (unsigned char)c) return d + i + 1;
    }
    return nullptr;
}

// ---------------------------------------------------------------- numbers
static __device__ int digit_val(int c) {
    if (c >= '0' && c <= '9') return c - '0';
    if (c >= 'a' && c <= 'z') return c - 'a' + 10;
    if (c >= 'A' && c <= 'Z') return c - 'A' + 10;
    return 99;
}

static __device__ unsigned long long parse_ull(const char* s, char** end, int base, bool* neg,
                                               bool* overflow) {
    const char* p = s;
    while (__gpu_isspace(*p)) p++;
    *neg = false;
    *overflow = false;
    if (*p == '+' || *p == '-') {
        *neg = *p == '-';
        p++;
    }
    if ((base == 0 || base == 16) && p[0] == '0' && (p[1] == 'x' || p[1] == 'X') &&
        digit_val(p[2]) < 16) {
        p += 2;
        base = 16;
    } else if (base == 0) {
        base = p[0] == '0' ? 8 : 10;
    }
    unsigned long long v = 0;
    const char* start = p;
    for (;; p++) {
        int d = digit_val(*p);
        if (d >= base) break;
        unsigned long long nv = v * base + d;
        if (nv / base != v && !*overflow) *overflow = true;
        v = nv;
    }
    if (end) *end = (char*)(p == start ? s : p);
    return v;
}

__device__ long long __gpu_strtoll(const char* nptr, char** endptr, int base) {
    bool neg, of;
    unsigned long long u = parse_ull(nptr, endptr, base, &neg, &of);
    if (of || (!neg && u > 0x7fffffffffffffffull)) return neg ? (-0x7fffffffffffffffll - 1) : 0x7fffffffffffffffll;
    if (neg && u > 0x8000000000000000ull) return -0x7fffffffffffffffll - 1;
    return neg ? (long long)(0ull - u) : (long long)u;
}
__device__ unsigned long long __gpu_strtoull(const char* nptr, char** endptr, int base) {
    bool neg, of;
    unsigned long long u = parse_ull(nptr, endptr, base, &neg, &of);
    if (of) return ~0ull;
    return neg ? 0ull - u : u;
}
__device__ long __gpu_strtol(const char* nptr, char** endptr, int base) {
    return (long)__gpu_strtoll(nptr, endptr, base);
}
__device__ unsigned long __gpu_strtoul(const char* nptr, char** endptr, int base) {
    return (unsigned long)__gpu_strtoull(nptr, endptr, base);
}
__device__ int __gpu_atoi(const char* nptr) { return (int)__gpu_strtol(nptr, nullptr, 10); }
__device__ long __gpu_atol(const char* nptr) { return __gpu_strtol(nptr, nullptr, 10); }
__device__ long long __gpu_atoll(const char* nptr) { return __gpu_strtoll(nptr, nullptr, 10); }

// Decimal to double.  Mantissas of up to 19 digits with |exponent| <= 22 are
// converted exactly (one rounding); other inputs by scaled multiplication.
__device__ double __gpu_strtod(const char* nptr, char** endptr) {
    const char* p = nptr;
    while (__gpu_isspace(*p)) p++;
    bool neg = false;
    if (*p == '+' || *p == '-') {
        neg = *p == '-';
        p++;
    }
    if ((p[0] | 32) == 'i' && (p[1] | 32) == 'n' && (p[2] | 32) == 'f') {
        p += 3;
        if ((p[0] | 32) == 'i' && (p[1] | 32) == 'n' && (p[2] | 32) == 'i' && (p[3] | 32) == 't' &&
            (p[4] | 32) == 'y')
            p += 5;
        if (endptr) *endptr = (char*)p;
        return neg ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff0000000000000ll);
    }
    if ((p[0] | 32) == 'n' && (p[1] | 32) == 'a' && (p[2] | 32) == 'n') {
        if (endptr) *endptr = (char*)(p + 3);
        return __longlong_as_double(0x7ff8000000000000ll);
    }
    unsigned long long mant = 0;
    int ndig = 0, dexp = 0;
    bool any = false;
    for (; *p >= '0' && *p <= '9'; p++) {
        any = true;
        if (ndig < 19) {
            mant = mant * 10 + (*p - '0');
            if (mant) ndig++;
        } else {
            dexp++;
        }
    }
    if (*p == '.') {
        p++;
        for (; *p >= '0' && *p <= '9'; p++) {
            any = true;
            if (ndig < 19) {
                mant = mant * 10 + (*p - '0');
                if (mant) ndig++;
                dexp--;
            }
        }
    }
    if (!any) {
        if (endptr) *endptr = (char*)nptr;
        return 0.0;
    }
    if (*p == 'e' || *p == 'E') {
        const char* q = p + 1;
        bool eneg = false;
        if (*q == '+' || *q == '-') {
            eneg = *q == '-';
            q++;
        }
        if (*q >= '0' && *q <= '9') {
            int e = 0;
            for (; *q >= '0' && *q <= '9'; q++)
                if (e < 100000) e = e * 10 + (*q - '0');
            dexp += eneg ? -e : e;
            p = q;
        }
    }
    if (endptr) *endptr = (char*)p;
    const double p10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                            1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    double v;
    if (mant < (1ull << 53) && dexp >= -22 && dexp <= 22) {
        v = (double)mant;
        v = dexp >= 0 ? v * p10[dexp] : v / p10[-dexp];
    } else {
        v = (double)mant;
        int e = dexp;
        while (e > 22) {
            v *= 1e22;
            e -= 22;
        }
        while (e < -22) {
            v /= 1e22;
            e += 22;
        }
        v = e >= 0 ? v * p10[e] : v / p10[-e];
    }
    return neg ? -v : v;
}
__device__ float __gpu_strtof(const char* nptr, char** endptr) {
    return (float)__gpu_strtod(nptr, endptr);
}
__device__ double __gpu_atof(const char* nptr) { return __gpu_strtod(nptr, nullptr); }

// ---------------------------------------------------------------- environment
__device__ char* __gpu_getenv(const char* name) {
    (void)name;
    return nullptr;
}
__device__ int* __gpu_errno_location(void) { return &bctx().priv->errno_v; }

__device__ int __gpu_gethostname(char* name, size_t len) {
    const char h[] = "gpumpi-gb300";
    size_t i = 0;
    for (; i + 1 < len && h[i]; i++) name[i] = h[i];
    if (len) name[i] = 0;
    return 0;
}
__device__ int __gpu_getpagesize(void) { return 4096; }

static __device__ void spin_ns(u64 ns) {
    u64 t0 = gtime();
    while (gtime() - t0 < ns) __nanosleep(1000);
}
__device__ unsigned int __gpu_sleep(unsigned int seconds) {
    spin_ns((u64)seconds * 1000000000ull);
    return 0;
}
__device__ int __gpu_usleep(unsigned int usec) {
    spin_ns((u64)usec * 1000ull);
    return 0;
}
__device__ int __gpu_gettimeofday(struct timeval* tv, void* tz) {
    (void)tz;
    u64 t = gtime();
    if (tv) {
        tv->tv_sec = (time_t)(t / 1000000000ull);
        tv->tv_usec = (suseconds_t)((t / 1000ull) % 1000000ull);
    }
    return 0;
}
__device__ time_t __gpu_time(time_t* tloc) {
    time_t t = (time_t)(gtime() / 1000000000ull);
    if (tloc) *tloc = t;
    return t;
}
__device__ clock_t __gpu_clock(void) { return (clock_t)(gtime() / 1000ull); }
__device__ int __gpu_omp_get_max_threads(void) { return 1; }
__device__ int __gpu_omp_get_num_threads(void) { return 1; }
__device__ int __gpu_omp_get_thread_num(void) { return 0; }
__device__ int __gpu_loop_block(void) { return bctx().cl_rank; }
__device__ double __gpu_omp_get_wtime(void) { return (double)gtime() * 1e-9; }

// POSIX getopt with per-rank state.
__device__ char** __gpu_optarg_location(void) { return &bctx().priv->opt_arg; }
__device__ int* __gpu_optind_location(void) { return &bctx().priv->opt_ind; }
__device__ int* __gpu_opterr_location(void) { return &bctx().priv->opt_err; }
__device__ int* __gpu_optopt_location(void) { return &bctx().priv->opt_opt; }

__device__ int __gpu_getopt(int argc, char* const argv[], const char* optstring) {
    RankPriv* p = bctx().priv;
    p->opt_arg = nullptr;
    if (p->opt_pos == 0) {
        if (p->opt_ind >= argc || !argv[p->opt_ind] || argv[p->opt_ind][0] != '-' ||
            argv[p->opt_ind][1] == 0)
            return -1;
        if (argv[p->opt_ind][1] == '-' && argv[p->opt_ind][2] == 0) {
            p->opt_ind++;
            return -1;
        }
        p->opt_pos = 1;
    }
    const char* arg = argv[p->opt_ind];
    int c = arg[p->opt_pos++];
    const char* spec = c == ':' ? nullptr : __gpu_strchr(optstring, c);
    if (!spec) {
        p->opt_opt = c;
        if (!arg[p->opt_pos]) {
            p->opt_ind++;
            p->opt_pos = 0;
        }
        return '?';
    }
    if (spec[1] == ':') {
        if (arg[p->opt_pos]) {
            p->opt_arg = (char*)&arg[p->opt_pos];
        } else if (p->opt_ind + 1 < argc) {
            p->opt_arg = argv[++p->opt_ind];
        } else {
            p->opt_opt = c;
            p->opt_ind++;
            p->opt_pos = 0;
            return optstring[0] == ':' ? ':' : '?';
        }
        p->opt_ind++;
        p->opt_pos = 0;
    } else if (!arg[p->opt_pos]) {
        p->opt_ind++;
        p->opt_pos = 0;
    }
    return c;
}
