// Device heap: a lock-free size-class slab allocator.
//
// The heap is a run of 64 KiB pages.  A page serves one size class
// (16 B << c, c = 0..11, i.e. 16 B .. 32 KiB) and tracks its chunks in a
// bitmap (1 = in use).  Allocation claims bits with atomicOr; when several
// lanes of a warp ask for the same class at once, the lowest lane claims a
// batch of bits for all of them in one atomic and hands them out (warp
// aggregation).  Free clears the bit with atomicAnd; a chunk's page and class
// follow from its address.  A claim scans a window of the class's pages from
// a per-SM-stripe hint; freed chunks outside that window are found through a
// per-class tagged (ABA-safe) stack of pages that have free chunks, onto which
// a free pushes its page unless it is already listed; only when both come up
// empty does a claim take a fresh page.  Requests above 32 KiB take runs of
// whole pages from one address-ordered list of free runs (first fit, split on
// allocation, merged with both neighbours on free) or, when no run fits, from
// the bump pointer (without the lock while no free run exists).  The list sits
// behind a test-and-test-and-set lock whose wait is bounded by the global timer
// (a wait that runs out returns NULL); a free walks the address-ordered list,
// so thousands of large frees at once serialise on it (see the allocator
// tests for the sizes covered).
//
// This replaces CUDA's device malloc (gpu_libs/gpu_libc/stdlib.cu:70-91) and
// the reference's experimental coalescing allocators (gpu_libs/gpu_malloc/*),
// whose measured cost this design targets: 13.4 M cycles per malloc for the
// CUDA heap at 12x1024 threads vs 0.17-3.3 M for the coalescing variants.
#include "rt.cuh"

namespace gm {

constexpr u32 PAGE = 64 * 1024;
constexpr int NCLS = 12;
constexpr int HINTS = 256;            // per-SM claim hints (SM ids are below 256)
constexpr int LINE_U64 = 16;          // one 128-byte line of u64 words
constexpr int LINE_U32 = 32;          // ... of u32 words
constexpr u32 CLS_LARGE = 0xFE;       // first page of an allocated large run
constexpr u32 CLS_FREE_RUN = 0xFD;    // first page of a free large run
constexpr u64 LOCK_WAIT_NS = 2000000000ull;
constexpr u32 NO_PAGE = 0xffffffffu;
constexpr int SCAN_PAGES = 64;

struct PageMeta {
    u32 cls;
    u32 npages;     // pages of a large run (first page only)
    u32 next;       // free-run list link: page + 1, 0 = end
    u32 slot;       // index of the page in its class list
    u32 pnext;      // partial-stack link: page + 1, 0 = end
    u32 listed;     // 1 while the page is on its class's partial stack
    u32 nfree;      // free chunks, never below the true count (frees add before
                    // clearing their bit, claims subtract after setting theirs)
    u32 pad;
    u64 bits[64];
};
static_assert(sizeof(PageMeta) % 8 == 0 && offsetof(PageMeta, bits) % 8 == 0, "64-bit atomics on bits");

// Partial-page stacks: heads hold (tag << 32) | (page + 1).
static __device__ void push_partial(Heap* h, int c, u32 p) {
    PageMeta* pm = &h->meta[p];
    if (atomicCAS(&pm->listed, 0u, 1u) != 0u) return;
    u64* head = &h->partial[c * LINE_U64];
    u64 old = *(volatile u64*)head;
    for (;;) {
        *(volatile u32*)&pm->pnext = (u32)(old & 0xffffffffull);
        __threadfence();
        const u64 nw = (((old >> 32) + 1) << 32) | (u64)(p + 1);
        const u64 seen = atomicCAS(head, old, nw);
        if (seen == old) return;
        old = seen;
    }
}

static __device__ u32 pop_partial(Heap* h, int c) {
    u64* head = &h->partial[c * LINE_U64];
    u64 old = *(volatile u64*)head;
    while ((old & 0xffffffffull) != 0) {
        const u32 cand = (u32)(old & 0xffffffffull) - 1;
        const u32 nxt = *(volatile u32*)&h->meta[cand].pnext;
        const u64 nw = (((old >> 32) + 1) << 32) | nxt;
        const u64 seen = atomicCAS(head, old, nw);
        if (seen == old) {
            atomicExch(&h->meta[cand].listed, 0u);
            return cand;
        }
        old = seen;
    }
    return 0xffffffffu;
}

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
                                     u64* m_out, u32* left = nullptr) {
    PageMeta* pm = &h->meta[p];
    if (*(volatile u32*)&pm->nfree == 0) return false;   // full: one load instead of a bitmap scan
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
                const u32 k = (u32)__popcll((long long)got);
                const u32 before = atomicSub(&pm->nfree, k);
                if (left) *left = before - k;
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
    const u32 n = *(volatile u32*)&h->cls_count[c * LINE_U32];
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
    // Pages whose chunks were freed outside the window.
    for (int tries = 0; tries < 16; tries++) {
        const u32 p = pop_partial(h, c);
        if (p == NO_PAGE) break;
        atomicAdd(&h->stats[4], 1u);
        u32 left = 0;
        if (claim_in_page(h, p, c, want, (int)(stripe % words_of(c)), w, m, &left)) {
            *hint = *(volatile u32*)&h->meta[p].slot;   // the window moves to a page with room
            if (left) push_partial(h, c, p);            // still room: keep it findable
            *page = p;
            return true;
        }
        atomicAdd(&h->stats[5], 1u);
    }
    // Fresh page from the bump pointer; its bitmap is still all zero.  Claim
    // this group's chunks before the page is published in the class list:
    // once listed, other warps may take its chunks, and a page of a large
    // class (16 or 32 chunks) could be drained before its creator claimed any.
    // (checked first, so a full heap does not keep moving the bump pointer:
    // it overshoots npages by at most the number of concurrent claimers)
    if (*(volatile u32*)h->next_page >= h->npages) return false;
    u32 p = atomicAdd(h->next_page, 1u);
    if (p >= h->npages) return false;
    atomicAdd(&h->stats[3], 1u);
    h->meta[p].cls = (u32)c;
    h->meta[p].nfree = chunks_of(c);
    u32 left = 0;
    if (!claim_in_page(h, p, c, want, 0, w, m, &left)) return false;
    __threadfence();
    u32 slot = atomicAdd(&h->cls_count[c * LINE_U32], 1u);
    h->meta[p].slot = slot;
    __threadfence();
    if (slot < h->npages) {
        ((volatile u32*)h->cls_pages)[(u64)c * h->npages + slot] = p;
        *hint = slot;
    }
    if (left) push_partial(h, c, p);   // other stripes find its room through the stack
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

// Test-and-test-and-set with exponential back-off: waiters read the lock word
// and try the CAS only when it looks free, so thousands of waiters do not
// queue atomics in front of the holder's release.
static __device__ bool large_lock(Heap* h) {
    if (atomicCAS(h->large_lock, 0u, 1u) != 0u) {
        const u64 t0 = gtime();
        unsigned ns = 64;
        for (;;) {
            if (*(volatile u32*)h->large_lock == 0u && atomicCAS(h->large_lock, 0u, 1u) == 0u) break;
            if (gtime() - t0 > LOCK_WAIT_NS) {
                atomicAdd(&h->stats[2], 1u);
                return false;
            }
            __nanosleep(ns);
            if (ns < 8192) ns <<= 1;
        }
    }
    __threadfence();
    return true;
}

// Fresh pages from the bump pointer need no lock (a failed request moves nothing).
static __device__ u32 large_bump(Heap* h, u32 n) {
    u32 first = *(volatile u32*)h->next_page;
    while ((u64)first + n <= h->npages) {
        const u32 seen = atomicCAS(h->next_page, first, first + n);
        if (seen == first) return first;
        first = seen;
    }
    return NO_PAGE;
}

static __device__ void large_unlock(Heap* h) {
    __threadfence();
    atomicExch(h->large_lock, 0u);
}

static __device__ void* large_alloc(Heap* h, u64 bytes) {
    const u64 n64 = (bytes + PAGE - 1) / PAGE;
    if (n64 > h->npages) return nullptr;
    const u32 n = (u32)n64;
    if (*(volatile u32*)h->large_head == 0) {
        // no free run to reuse: take fresh pages without the lock (the pages
        // of a fresh run belong to this caller alone, so are its page records)
        const u32 p = large_bump(h, n);
        if (p != NO_PAGE) {
            h->meta[p].npages = n;
            h->meta[p].cls = CLS_LARGE;
            __threadfence();
            return h->base + (u64)p * PAGE;
        }
    }
    if (!large_lock(h)) return nullptr;
    volatile PageMeta* meta = h->meta;
    u32 p = NO_PAGE;
    u32 prev = NO_PAGE;
    u32 cur = *(volatile u32*)h->large_head;   // page + 1
    while (cur) {
        const u32 c = cur - 1;
        const u32 len = meta[c].npages;
        const u32 nxt = meta[c].next;
        if (len >= n) {
            u32 link = nxt;
            if (len > n) {                   // split: the tail stays free
                const u32 rest = c + n;
                meta[rest].cls = CLS_FREE_RUN;
                meta[rest].npages = len - n;
                meta[rest].next = nxt;
                link = rest + 1;
            }
            if (prev == NO_PAGE) *(volatile u32*)h->large_head = link;
            else meta[prev].next = link;
            p = c;
            break;
        }
        prev = c;
        cur = nxt;
    }
    if (p == NO_PAGE) p = large_bump(h, n);   // only when the run fits
    if (p != NO_PAGE) {
        meta[p].cls = CLS_LARGE;
        meta[p].npages = n;
    }
    large_unlock(h);
    return p == NO_PAGE ? nullptr : h->base + (u64)p * PAGE;
}

// Return a large run to the free list, merged with free neighbours.
static __device__ void large_release(Heap* h, u32 p) {
    if (!large_lock(h)) return;               // counted in stats[2]; the run is lost
    volatile PageMeta* meta = h->meta;
    u32 n = meta[p].npages;
    u32 prev = NO_PAGE;
    u32 cur = *(volatile u32*)h->large_head;
    while (cur && cur - 1 < p) {
        prev = cur - 1;
        cur = meta[prev].next;
    }
    u32 link = cur;
    if (cur && p + n == cur - 1) {            // merge with the next free run
        n += meta[cur - 1].npages;
        link = meta[cur - 1].next;
        meta[cur - 1].cls = 0;
    }
    if (prev != NO_PAGE && prev + meta[prev].npages == p) {   // merge into the previous run
        meta[prev].npages = meta[prev].npages + n;
        meta[prev].next = link;
        meta[p].cls = 0;
    } else {
        meta[p].cls = CLS_FREE_RUN;
        meta[p].npages = n;
        meta[p].next = link;
        if (prev == NO_PAGE) *(volatile u32*)h->large_head = p + 1;
        else meta[prev].next = p + 1;
    }
    large_unlock(h);
}

__device__ void* heap_alloc(Heap* h, u64 bytes) {
    if (h == nullptr || h->base == nullptr) return nullptr;
    if (bytes == 0) bytes = 1;
    if (bytes > (PAGE >> 1)) return large_alloc(h, bytes);
    void* p = small_alloc(h, class_of(bytes));

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
        const u32 word = (u32)(chunk / 64);
        const u64 bit = 1ull << (chunk % 64);
        // Lanes of a warp freeing chunks of the same bitmap word free them
        // together: one fence and one atomicAnd for the group, by its lowest lane.
        const unsigned act = __activemask();
        const unsigned grp = __match_any_sync(act, ((unsigned long long)p << 8) | word);
        const unsigned lo = __reduce_or_sync(grp, (unsigned)bit);
        const unsigned hi = __reduce_or_sync(grp, (unsigned)(bit >> 32));
        __syncwarp(grp);   // orders every lane's last use of its chunk before the leader's release
        if ((int)(threadIdx.x & 31) != __ffs(grp) - 1) return;
        // release: the group's chunks can be claimed again only after this
        __threadfence();
        atomicAdd(&pm->nfree, (u32)__popc(grp));
        atomicAnd(&pm->bits[word], ~(((u64)hi << 32) | lo));
        if (*(volatile u32*)&pm->listed == 0u) push_partial(h, (int)cls, p);
        return;
    }
    if (cls == CLS_LARGE) {
        if ((off % PAGE) != 0) {
            atomicAdd(&h->stats[1], 1u);
            return;
        }
        large_release(h, p);
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

// Control words of a heap, in one zero-initialised block: the tagged heads of
// the partial-page stacks, the class page counts, the per-stripe hints, the
// bump pointer, the free-run list head and lock, and the statistics
// (1 frees of foreign pointers, 2 lock waits that ran out, 3 fresh small
// pages, 4 partial-stack pops, 5 pops that found the page full).
// Control words of a heap.  Every word that many threads update atomically
// (each class's partial-stack head and page count, the bump pointer, the
// large-run lock and list head, the counters) has a 128-byte line of its own,
// so that atomics on one do not queue behind atomics on another.
constexpr size_t LINE = 128;
constexpr size_t CTL_PARTIAL = 0;
constexpr size_t CTL_COUNT = CTL_PARTIAL + LINE * NCLS;
constexpr size_t CTL_HINT = CTL_COUNT + LINE * NCLS;
constexpr size_t CTL_NEXT = CTL_HINT + ((sizeof(u32) * NCLS * HINTS + LINE - 1) / LINE) * LINE;
constexpr size_t CTL_LARGE_HEAD = CTL_NEXT + LINE;
constexpr size_t CTL_LARGE_LOCK = CTL_LARGE_HEAD + LINE;
constexpr size_t CTL_STATS = CTL_LARGE_LOCK + LINE;
constexpr size_t CTL_BYTES = (CTL_STATS + sizeof(u32) * 8 + 255) & ~(size_t)255;

__host__ size_t heap_ctl_bytes() { return CTL_BYTES; }

__host__ void heap_set_ctl(Heap& h, char* ctl) {
    h.large_head = (u32*)(ctl + CTL_LARGE_HEAD);
    h.large_lock = (u32*)(ctl + CTL_LARGE_LOCK);
    h.partial = (u64*)(ctl + CTL_PARTIAL);
    h.cls_count = (u32*)(ctl + CTL_COUNT);
    h.cls_hint = (u32*)(ctl + CTL_HINT);
    h.next_page = (u32*)(ctl + CTL_NEXT);
    h.stats = (u32*)(ctl + CTL_STATS);
}

}  // namespace gm

// Size of the allocator's per-page metadata, for the host-side heap set-up.
extern "C" __host__ size_t gpumpi_heap_meta_bytes() { return sizeof(gm::PageMeta); }
