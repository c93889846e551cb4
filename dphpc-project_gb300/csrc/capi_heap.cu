// Allocator churn: every thread of a grid loops malloc, fill, verify, free.
//
// This is the allocation workload of converted programs taken to its limit:
// the reference's device malloc (CUDA's heap behind __gpu_malloc,
// gpu_libs/gpu_libc/stdlib.cu:70-91) measured 13.4 M cycles per call at
// 12x1024 threads, which is what the slab allocator in gmalloc.cu replaces.
// Each thread keeps up to `live` objects, draws sizes floor(2^U) bytes with
// U uniform in [4, 12) (log-uniform 16 B .. 4 KiB), writes a pattern derived
// from (thread, iteration) over the whole object and checks it before the
// object is freed.  Failed allocations, corrupted patterns and misaligned
// pointers are counted; the latency of every malloc call (SM clock cycles)
// goes into a histogram of 4 buckets per octave.
//
// cuda_heap = 1 runs the same loop on CUDA's device malloc/free for
// comparison (the allocator the reference used).
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "gpumpi.h"
#include "hostjob.h"
#include "rt.cuh"

using namespace gm;

extern "C" size_t gpumpi_heap_meta_bytes();

namespace {

constexpr int CHURN_MAX_LIVE = 16;
constexpr int HIST_BUCKETS = 256;

struct ChurnArgs {
    Heap* heap;
    int iters;
    int live;
    int cuda_heap;
    unsigned fixed_bytes;        // 0: log-uniform sizes; else every object has this size
    unsigned long long seed;
    unsigned int* hist;          // [HIST_BUCKETS] malloc latency
    unsigned int* fhist;         // [HIST_BUCKETS] free latency
    unsigned long long* count;   // allocs, frees, failed, corrupt, misaligned, malloc cycles, free cycles
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ int bucket_of(unsigned long long v) {
    if (v < 4) return (int)v;
    const int lg = 63 - __clzll((long long)v);
    return lg * 4 + (int)((v >> (lg - 2)) & 3);
}

__device__ void fill(unsigned char* p, unsigned n, unsigned tag) {
    unsigned* w = (unsigned*)p;
    const unsigned nw = n / 4;
    for (unsigned i = 0; i < nw; i++) w[i] = tag ^ (i * 0x9E3779B1u);
    for (unsigned i = nw * 4; i < n; i++) p[i] = (unsigned char)(tag >> (8 * (i & 3)));
}

__device__ bool check(const unsigned char* p, unsigned n, unsigned tag) {
    const unsigned* w = (const unsigned*)p;
    const unsigned nw = n / 4;
    bool ok = true;
    for (unsigned i = 0; i < nw; i++) ok &= w[i] == (tag ^ (i * 0x9E3779B1u));
    for (unsigned i = nw * 4; i < n; i++) ok &= p[i] == (unsigned char)(tag >> (8 * (i & 3)));
    return ok;
}

// Two instances: CUDA sizes its device heap only before the first launch of a
// kernel that contains a malloc call, so the slab arm must not contain one.
template <bool CUDA_HEAP>
__global__ void __launch_bounds__(1024) gpumpi_churn_kernel(ChurnArgs a) {
    __shared__ unsigned int hist[HIST_BUCKETS];
    __shared__ unsigned int fhist[HIST_BUCKETS];
    __shared__ unsigned long long cnt[7];
    for (int i = threadIdx.x; i < HIST_BUCKETS; i += blockDim.x) {
        hist[i] = 0;
        fhist[i] = 0;
    }
    if (threadIdx.x < 7) cnt[threadIdx.x] = 0;
    __syncthreads();
    const unsigned long long tid = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long rng = mix64(a.seed ^ (tid * 0x9e3779b97f4a7c15ull));
    unsigned char* ring[CHURN_MAX_LIVE] = {};
    unsigned size[CHURN_MAX_LIVE] = {};
    unsigned tag[CHURN_MAX_LIVE] = {};
    int head = 0, n = 0;
    unsigned long long allocs = 0, frees = 0, failed = 0, corrupt = 0, misaligned = 0, mcyc = 0, fcyc = 0;
    auto release = [&](int k) {
        if (!check(ring[k], size[k], tag[k])) corrupt++;
        const long long t0 = clock64();
        if (CUDA_HEAP) free(ring[k]);
        else heap_free(a.heap, ring[k]);
        const long long dt = clock64() - t0;
        atomicAdd(&fhist[bucket_of((unsigned long long)(dt > 0 ? dt : 0))], 1u);
        fcyc += (unsigned long long)(dt > 0 ? dt : 0);
        frees++;
    };
    for (int it = 0; it < a.iters; it++) {
        if (n == a.live) {
            release(head);
            head = (head + 1) % a.live;
            n--;
        }
        rng += 0x9e3779b97f4a7c15ull;
        const unsigned long long r = mix64(rng);
        const double u = (double)(r >> 11) * (1.0 / 9007199254740992.0);   // [0, 1)
        unsigned bytes = (unsigned)exp2(4.0 + 8.0 * u);
        if (bytes > 4095) bytes = 4095;
        if (a.fixed_bytes) bytes = a.fixed_bytes;
        const long long t0 = clock64();
        unsigned char* p = CUDA_HEAP ? (unsigned char*)malloc(bytes) : (unsigned char*)heap_alloc(a.heap, bytes);
        const long long dt = clock64() - t0;
        atomicAdd(&hist[bucket_of((unsigned long long)(dt > 0 ? dt : 0))], 1u);
        mcyc += (unsigned long long)(dt > 0 ? dt : 0);
        allocs++;
        if (!p) {
            failed++;
            continue;
        }
        if ((unsigned long long)p & 15) misaligned++;
        const int k = (head + n) % a.live;
        ring[k] = p;
        size[k] = bytes;
        tag[k] = (unsigned)mix64(tid * 1000003ull + (unsigned long long)it);
        fill(p, bytes, tag[k]);
        n++;
    }
    while (n > 0) {
        release(head);
        head = (head + 1) % a.live;
        n--;
    }
    atomicAdd(&cnt[0], allocs);
    atomicAdd(&cnt[1], frees);
    atomicAdd(&cnt[2], failed);
    atomicAdd(&cnt[3], corrupt);
    atomicAdd(&cnt[4], misaligned);
    atomicAdd(&cnt[5], mcyc);
    atomicAdd(&cnt[6], fcyc);
    __syncthreads();
    for (int i = threadIdx.x; i < HIST_BUCKETS; i += blockDim.x) {
        if (hist[i]) atomicAdd(&a.hist[i], hist[i]);
        if (fhist[i]) atomicAdd(&a.fhist[i], fhist[i]);
    }
    if (threadIdx.x < 7) atomicAdd(&a.count[threadIdx.x], cnt[threadIdx.x]);
}

// Lower edge of a histogram bucket, in cycles.
unsigned long long bucket_floor(int b) {
    if (b < 4) return (unsigned long long)b;
    const int lg = b / 4, sub = b % 4;
    return (1ull << lg) + ((unsigned long long)sub << (lg - 2));
}

unsigned long long percentile(const unsigned long long* h, double q) {
    unsigned long long total = 0;
    for (int i = 0; i < HIST_BUCKETS; i++) total += h[i];
    if (!total) return 0;
    const double want = q * (double)total;
    unsigned long long acc = 0;
    for (int i = 0; i < HIST_BUCKETS; i++) {
        acc += h[i];
        if ((double)acc >= want) return bucket_floor(i);
    }
    return bucket_floor(HIST_BUCKETS - 1);
}

#define HK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[300];                                                                 \
            snprintf(m_, sizeof(m_), "%s: %s", #call, cudaGetErrorString(e_));            \
            set_last_error(m_);                                                           \
            rc = GPUMPI_ECUDA;                                                            \
            goto done;                                                                    \
        }                                                                                 \
    } while (0)

}  // namespace

static int churn_run(int blocks, int threads, int iters, int live, uint64_t seed, size_t heap_bytes,
                     int cuda_heap, unsigned fixed_bytes, void* stream, gpumpi_churn_stats* out);

extern "C" int gpumpi_malloc_churn(int blocks, int threads, int iters, int live, uint64_t seed,
                                   size_t heap_bytes, int cuda_heap, void* stream, gpumpi_churn_stats* out) {
    if (!out || blocks < 1 || threads < 32 || threads > 1024 || threads % 32 || iters < 0 || live < 1 ||
        live > CHURN_MAX_LIVE) {
        set_last_error("gpumpi_malloc_churn: bad arguments (live must be 1..16, threads 32..1024)");
        return GPUMPI_EINVAL;
    }
    return churn_run(blocks, threads, iters, live, seed, heap_bytes, cuda_heap, 0, stream, out);
}

extern "C" int gpumpi_malloc_bench(int blocks, int threads, size_t bytes, size_t heap_bytes, int cuda_heap,
                                   void* stream, gpumpi_churn_stats* out) {
    if (!out || blocks < 1 || threads < 32 || threads > 1024 || threads % 32 || bytes < 1 || bytes > (1u << 20)) {
        set_last_error("gpumpi_malloc_bench: bad arguments (threads 32..1024, bytes 1..1 MiB)");
        return GPUMPI_EINVAL;
    }
    return churn_run(blocks, threads, 1, 1, 1, heap_bytes, cuda_heap, (unsigned)bytes, stream, out);
}

static int churn_run(int blocks, int threads, int iters, int live, uint64_t seed, size_t heap_bytes,
                     int cuda_heap, unsigned fixed_bytes, void* stream, gpumpi_churn_stats* out) {
    if (heap_bytes == 0) heap_bytes = (size_t)4 << 30;
    memset(out, 0, sizeof(*out));
    int rc = GPUMPI_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned npages = (unsigned)((heap_bytes + 65535) / 65536);
    const size_t meta = gpumpi_heap_meta_bytes() * npages;
    const size_t ctl = heap_ctl_bytes();
    const size_t clsp = sizeof(u32) * 12 * (size_t)npages;
    // Side regions, each at a 256-byte boundary: the Heap struct, the latency
    // histogram, the counters, the allocator's control words, the page
    // metadata (64-bit bitmaps updated with 64-bit atomics) and the page lists.
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t o_hist = al(sizeof(Heap));
    const size_t o_fhist = al(o_hist + HIST_BUCKETS * sizeof(unsigned));
    const size_t o_cnt = al(o_fhist + HIST_BUCKETS * sizeof(unsigned));
    const size_t o_ctl = al(o_cnt + 8 * sizeof(unsigned long long));
    const size_t o_meta = al(o_ctl + ctl);
    const size_t o_clsp = al(o_meta + meta);
    const size_t small = al(o_clsp + clsp);
    char* mem = nullptr;
    char* heap_mem = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    unsigned hist32[HIST_BUCKETS], fhist32[HIST_BUCKETS];
    unsigned long long hist[HIST_BUCKETS], fhist[HIST_BUCKETS], cnt[7];
    float ms = 0;
    Heap h;
    ChurnArgs a;
    memset(&h, 0, sizeof(h));
    HK(cudaMalloc(&mem, small));
    if (!cuda_heap) HK(cudaMalloc(&heap_mem, (size_t)npages * 65536));
    HK(cudaMemsetAsync(mem, 0, o_clsp, st));
    HK(cudaMemsetAsync(mem + o_clsp, 0xff, clsp, st));
    {
        Heap* dh = (Heap*)mem;
        unsigned* dhist = (unsigned*)(mem + o_hist);
        unsigned long long* dcnt = (unsigned long long*)(mem + o_cnt);
        h.base = heap_mem;
        h.bytes = cuda_heap ? 0 : (u64)npages * 65536;
        h.npages = cuda_heap ? 0 : npages;
        h.meta = (PageMeta*)(mem + o_meta);
        heap_set_ctl(h, mem + o_ctl);
        h.cls_pages = (u32*)(mem + o_clsp);
        if ((uintptr_t)h.meta % 8 || (uintptr_t)h.partial % 8 ||
            (uintptr_t)dcnt % 8 || (uintptr_t)heap_mem % 16) {
            set_last_error("gpumpi_malloc_churn: internal layout misaligned");
            rc = GPUMPI_EINVAL;
            goto done;
        }
        HK(cudaMemcpyAsync(dh, &h, sizeof(Heap), cudaMemcpyHostToDevice, st));
        a.heap = dh;
        a.iters = iters;
        a.live = live;
        a.cuda_heap = cuda_heap;
        a.seed = seed;
        a.fixed_bytes = fixed_bytes;
        a.hist = dhist;
        a.fhist = (unsigned*)(mem + o_fhist);
        a.count = dcnt;
    }
    if (cuda_heap) {
        // Size CUDA's device heap; refused once the CUDA-heap instance has run in this
        // context, in which case the current size stays.
        if (cudaDeviceSetLimit(cudaLimitMallocHeapSize, heap_bytes) != cudaSuccess) cudaGetLastError();
    }
    HK(cudaEventCreate(&e0));
    HK(cudaEventCreate(&e1));
    HK(cudaEventRecord(e0, st));
    if (cuda_heap) gpumpi_churn_kernel<true><<<blocks, threads, 0, st>>>(a);
    else gpumpi_churn_kernel<false><<<blocks, threads, 0, st>>>(a);
    HK(cudaGetLastError());
    HK(cudaEventRecord(e1, st));
    HK(cudaStreamSynchronize(st));
    HK(cudaEventElapsedTime(&ms, e0, e1));
    HK(cudaMemcpy(hist32, a.hist, sizeof(hist32), cudaMemcpyDeviceToHost));
    HK(cudaMemcpy(fhist32, a.fhist, sizeof(fhist32), cudaMemcpyDeviceToHost));
    HK(cudaMemcpy(cnt, a.count, sizeof(cnt), cudaMemcpyDeviceToHost));
    for (int i = 0; i < HIST_BUCKETS; i++) {
        hist[i] = hist32[i];
        fhist[i] = fhist32[i];
    }
    out->allocs = cnt[0];
    out->frees = cnt[1];
    out->failed = cnt[2];
    out->corrupt = cnt[3];
    out->misaligned = cnt[4];
    out->seconds = ms / 1000.0;
    out->ops_per_s = ms > 0 ? (double)(cnt[0] + cnt[1]) / (ms / 1000.0) : 0.0;
    out->malloc_cycles_p50 = percentile(hist, 0.50);
    out->malloc_cycles_p99 = percentile(hist, 0.99);
    out->malloc_cycles_mean = cnt[0] ? cnt[5] / cnt[0] : 0;
    out->free_cycles_p50 = percentile(fhist, 0.50);
    out->free_cycles_p99 = percentile(fhist, 0.99);
    out->free_cycles_mean = cnt[1] ? cnt[6] / cnt[1] : 0;
    if (!cuda_heap) {
        unsigned st8[8];
        HK(cudaMemcpy(st8, h.stats, sizeof(st8), cudaMemcpyDeviceToHost));
        out->fresh_pages = st8[3];
        out->partial_pops = st8[4];
        out->partial_full = st8[5];
    }
done:
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (heap_mem) cudaFree(heap_mem);
    if (mem) cudaFree(mem);
    return rc;
}
