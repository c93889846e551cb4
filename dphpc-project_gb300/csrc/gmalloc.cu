// Device heap: a lock-free size-class slab allocator.
//
// The heap is a run of 64 KiB pages.  A page serves one size class
// (16 B << c, c = 0..11, i.e. 16 B .. 32 KiB) and tracks its chunks in a
// bitmap (1 = in use).  Allocation claims bits with atomicOr; when several
// lanes of a warp ask for the same class at once, the lowest lane claims a
// batch of bits for all of them in one atomic and hands them out (warp
// aggregation).  Free clears the bit with atomicAnd; a chunk's page and class
// follow from its address.  Requests above 32 KiB take whole pages: exact-size
// runs of fewer than 64 pages are recycled through tagged (ABA-safe) stacks,
// longer runs come from the bump pointer and are not recycled.
//
// This replaces CUDA's device malloc (gpu_libs/gpu_libc/stdlib.cu:70-91) and
// the reference's experimental coalescing allocators (gpu_libs/gpu_malloc/*),
// whose measured cost this design targets: 13.4 M cycles per malloc for the
// CUDA heap at 12x1024 threads vs 0.17-3.3 M for the coalescing variants.
#include "rt.cuh"

namespace gm {

constexpr u32 PAGE = 64 * 1024;
constexpr int NCLS = 12;
constexpr int HINTS = 32;
constexpr int LARGE_BUCKETS = 64;
constexpr u32 CLS_LARGE = 0xFE;
constexpr u32 NO_PAGE = 0xffffffffu;
constexpr int SCAN_PAGES = 64;

struct PageMeta {
    u32 cls;
    u32 npages;
    u32 next;       // large free-list link: page + 1, 0 = end
    u32 pad;
    u64 bits[64];
};

static __device__ __forceinline__ int class_of(u64 bytes) {
    if (bytes <= 16) return 0;
    int c = 64 - __clzll((long long)(bytes - 1)) - 4;
    return c;
}
static __device__ __forceinline__ u32 chunks_of(int c) { return 4096u >> c; }
static __device__ __forceinline__ int words_of(int c) {
    u32 n = chunks_of(c);
    return n >= 64 ? (int)(n / 64) : 1;
}
static __device__ __forceinline__ u64 valid_mask(int c) {
    u32 n = chunks_of(c);
    return n >= 64 ? ~0ull : ((1ull << n) - 1);
}

static __device__ __forceinline__ u64 lowest_bits(u64 m, int k) {
    u64 pick = 0;
    for (int i = 0; i < k && m; i++) {
        u64 low = m & (~m + 1);
        pick |= low;
        m ^= low;
    }
    return pick;
}

static __device__ __forceinline__ int nth_set_bit(u64 m, int n) {
    for (int i = 0; i < n; i++) m &= m - 1;
    return __ffsll((long long)m) - 1;
}

static __device__ __forceinline__ u32 smid() {
    u32 id;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(id));
    return id;
}

// Try to claim up to `want` chunks of class c from page p.
static __device__ bool claim_in_page(Heap* h, u32 p, int c, int want, int rot, int* w_out,
                                     u64* m_out) {
    PageMeta* pm = &h->meta[p];
    const int nw = words_of(c);
    const u64 valid = valid_mask(c);
    for (int k = 0; k < nw; k++) {
        int w = (k + rot) % nw;
        u64 used = *(volatile u64*)&pm->bits[w];
        u64 freeb = ~used & valid;
        while (freeb) {
            u64 pick = lowest_bits(freeb, want);
            u64 old = atomicOr(&pm->bits[w], pick);
            u64 got = pick & ~old;
            if (got) {
                __threadfence();
                *w_out = w;
                *m_out = got;
                return true;
            }
            freeb = ~(old | pick) & valid;
        }
    }
    return false;
}

// Leader of a warp group: claim a batch of chunks of class c.
static __device__ bool claim_batch(Heap* h, int c, int want, u32* page, int* w, u64* m) {
    const int stripe = (int)(smid() % HINTS);
    u32* hint = &h->cls_hint[c * HINTS + stripe];
    const u32 n = *(volatile u32*)&h->cls_count[c];
    const u32* list = h->cls_pages + (u64)c * h->npages;
    if (n > 0) {
        u32 start = *(volatile u32*)hint % n;
        const u32 scan = n < SCAN_PAGES ? n : SCAN_PAGES;
        for (u32 k = 0; k < scan; k++) {
            u32 idx = (start + k) % n;
            u32 p = *(volatile const u32*)&list[idx];
            if (p == NO_PAGE) continue;
            if (claim_in_page(h, p, c, want, (int)(stripe % words_of(c)), w, m)) {
                if (idx != start) *hint = idx;
                *page = p;
                return true;
            }
        }
    }
    // Fresh page from the bump pointer; its bitmap is still all zero.
    u32 p = atomicAdd(h->next_page, 1u);
    if (p >= h->npages) return false;
    h->meta[p].cls = (u32)c;
    __threadfence();
    u32 slot = atomicAdd(&h->cls_count[c], 1u);
    if (slot < h->npages) {
        ((volatile u32*)h->cls_pages)[(u64)c * h->npages + slot] = p;
        *hint = slot;
    }
    if (!claim_in_page(h, p, c, want, 0, w, m)) return false;
    *page = p;
    return true;
}

static __device__ void* small_alloc(Heap* h, int c) {
    const unsigned active = __activemask();
    const unsigned grp = __match_any_sync(active, c);
    const int lane = (int)(threadIdx.x & 31);
    const int leader = __ffs(grp) - 1;
    const int rank_in = __popc(grp & ((1u << lane) - 1));
    const int need = __popc(grp);
    void* result = nullptr;
    int got = 0;
    while (got < need) {
        u32 page = 0;
        int w = 0;
        u64 m = 0;
        if (lane == leader) {
            if (!claim_batch(h, c, need - got, &page, &w, &m)) m = 0;
        }
        page = __shfl_sync(grp, page, leader);
        w = __shfl_sync(grp, w, leader);
        m = __shfl_sync(grp, m, leader);
        if (m == 0) break;
        const int k = __popcll((long long)m);
        const int idx = rank_in - got;
        if (idx >= 0 && idx < k) {
            const int bit = nth_set_bit(m, idx);
            const u64 chunk = (u64)w * 64 + bit;
            result = h->base + (u64)page * PAGE + (chunk << (4 + c));
        }
        got += k;
    }
    return result;
}

static __device__ void* large_alloc(Heap* h, u64 bytes) {
    const u64 n64 = (bytes + PAGE - 1) / PAGE;
    if (n64 > h->npages) return nullptr;
    const u32 n = (u32)n64;
    u32 p = NO_PAGE;
    if (n < LARGE_BUCKETS) {
        u64* head = &h->large_free[n];
        u64 old = *(volatile u64*)head;
        while ((old & 0xffffffffull) != 0) {
            u32 cand = (u32)(old & 0xffffffffull) - 1;
            u32 nxt = *(volatile u32*)&h->meta[cand].next;
            u64 nw = (((old >> 32) + 1) << 32) | nxt;
            u64 seen = atomicCAS(head, old, nw);
            if (seen == old) {
                p = cand;
                break;
            }
            old = seen;
        }
    }
    if (p == NO_PAGE) {
        u32 first = atomicAdd(h->next_page, n);
        if ((u64)first + n > h->npages) return nullptr;
        p = first;
    }
    h->meta[p].cls = CLS_LARGE;
    h->meta[p].npages = n;
    __threadfence();
    return h->base + (u64)p * PAGE;
}

__device__ void* heap_alloc(Heap* h, u64 bytes) {
    if (h == nullptr || h->base == nullptr) return nullptr;
    if (bytes == 0) bytes = 1;
    if (bytes > (PAGE >> 1)) return large_alloc(h, bytes);
    void* p = small_alloc(h, class_of(bytes));
    if (p) atomicAdd(&h->stats[0], 1u);
    return p;
}

__device__ void heap_free(Heap* h, void* ptr) {
    if (ptr == nullptr || h == nullptr) return;
    const u64 off = (u64)((char*)ptr - h->base);
    if ((char*)ptr < h->base || off >= h->bytes) {
        atomicAdd(&h->stats[1], 1u);  // foreign pointer: counted, ignored
        return;
    }
    const u32 p = (u32)(off / PAGE);
    PageMeta* pm = &h->meta[p];
    const u32 cls = *(volatile u32*)&pm->cls;
    if (cls < NCLS) {
        const u64 chunk = (off % PAGE) >> (4 + cls);
        __threadfence();
        atomicAnd(&pm->bits[chunk / 64], ~(1ull << (chunk % 64)));
        return;
    }
    if (cls == CLS_LARGE) {
        const u32 n = pm->npages;
        if (n >= LARGE_BUCKETS || (off % PAGE) != 0) return;
        u64* head = &h->large_free[n];
        u64 old = *(volatile u64*)head;
        for (;;) {
            pm->next = (u32)(old & 0xffffffffull);
            __threadfence();
            u64 nw = (((old >> 32) + 1) << 32) | (u64)(p + 1);
            u64 seen = atomicCAS(head, old, nw);
            if (seen == old) break;
            old = seen;
        }
        return;
    }
    atomicAdd(&h->stats[1], 1u);
}

__device__ u64 heap_usable_size(Heap* h, void* ptr) {
    if (ptr == nullptr) return 0;
    const u64 off = (u64)((char*)ptr - h->base);
    if ((char*)ptr < h->base || off >= h->bytes) return 0;
    const PageMeta* pm = &h->meta[off / PAGE];
    if (pm->cls < NCLS) return 16ull << pm->cls;
    if (pm->cls == CLS_LARGE) return (u64)pm->npages * PAGE;
    return 0;
}

}  // namespace gm

// Size of the allocator's per-page metadata, for the host-side heap set-up.
extern "C" __host__ size_t gpumpi_heap_meta_bytes() { return sizeof(gm::PageMeta); }
