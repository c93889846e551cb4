// Collective engine.  Every collective is a direct-pull schedule over one
// GPU's HBM: a rank publishes the addresses of its buffers in the
// communicator's table, raises its `arrive` flag, and the ranks that need the
// data copy (or reduce) it straight out of the owner's buffer with all threads
// of their block.  A rank whose buffers others read waits on their `depart`
// flags before returning, so MPI buffer semantics hold without any staging
// copy.  Flags carry the collective's sequence number on the communicator and
// are written only by their owner (no atomic read-modify-write anywhere).
//
// Reductions fold in rank order, acc = x_0; acc = op(x_q, acc) for q = 1..P-1,
// which is the order of the reference's generic MPI_Reduce
// (gpu_libs/gpu_mpi/mpi.cu:209-225, operators.cu:216-218).  Results are
// therefore bit-identical to a linear host reduction for every datatype,
// including FP64.  Work is split by element ranges, not by ranks, so the fold
// order of each element never changes.
//
// The reference's schedules were flat Send/Recv fan-outs from the root
// (mpi.cu:120-137, :291-322, :363-408, :484-591) and an atomicAdd reduction on
// MPI_COMM_WORLD (mpi.cu:148-179); the results here equal those of its rank-
// order paths.
#include "rt.cuh"

namespace gm {

constexpr u64 REDUCE_ROOT_ONLY_BYTES = 64 * 1024;     // total input bytes
constexpr u64 ALLREDUCE_DIRECT_BYTES = 16 * 1024;     // per-rank bytes
constexpr u64 WARP_COPY_BYTES = 16 * 1024;            // per-block copies below this go warp-parallel
constexpr u64 TINY_BLOCK_BYTES = 128;                 // ... and below this one block per thread

// Start a collective: thread 0 bumps the communicator's sequence number and
// publishes a view of the communicator to the block (bctx().cv).
static __device__ __forceinline__ u64 coll_begin(MPI_Comm_impl* c, int tid) {
    BlockCtx& b = bctx();
    bsync();
    if (tid == 0) {
        CommShared* s = c->cs;
        b.cv.shared = s;
        b.cv.pub = s->pub;
        b.cv.arrive = s->arrive;
        b.cv.mid = s->mid;
        b.cv.depart = s->depart;
        b.cv.P = c->size;
        b.cv.me = c->rank;
        b.cv.seq = ++c->seq;
    }
    bsync();
    return b.cv.seq;
}

static __device__ __forceinline__ void publish(MPI_Comm_impl* c, u64 seq, const Pub& p, int tid) {
    if (tid == 0) {
        c->cs->pub[c->rank] = p;
        __threadfence();
        st_release(&c->cs->arrive[c->rank], seq);
    }
}

static __device__ __forceinline__ void raise_flag(u64* flags, int me, u64 seq, int tid) {
    bsync();
    if (tid == 0) {
        __threadfence();
        st_release(&flags[me], seq);
    }
}

static __device__ __forceinline__ int wait_one(const u64* flags, int q, u64 seq, int tid) {
    int rc = 0;
    if (tid == 0) rc = wait_ge(&flags[q], seq);
    return (int)bcast(rc, tid);
}

// Elements per rank segment of an n-element reduction over P ranks: a whole
// number of 16-byte vectors, and of 128-byte lines once a segment is at least
// SEG_LINE_MIN_BYTES, so that no line of an input or an output is split
// between two ranks' segments (a line written in two parts at different times
// can be written back to DRAM twice, and one read in two parts fetched twice).
constexpr u64 SEG_LINE_MIN_BYTES = 4096;
static __device__ __forceinline__ u64 seg_len(u64 n, int P, int es) {
    u64 per = (n + P - 1) / P;
    const u64 vec = es < 16 ? 16 / es : 1;
    const u64 line = es < 128 ? 128 / es : 1;
    const u64 unit = per * (u64)es >= SEG_LINE_MIN_BYTES ? line : vec;
    per = (per + unit - 1) / unit * unit;
    return per;
}

// Copy nb blocks.  src(q)/dst(q)/bytes(q) come from the functor.  mode 1:
// blocks one after another, each by the whole thread block; mode 2: one block
// per warp, warps in parallel; mode 3: thread 0 streams every 16-byte aligned
// block through the bulk engine in one pipeline while the other threads wait,
// then all threads copy unaligned blocks and sub-16-byte tails; mode 0: mode 3
// for blocks of BULK_SEG_MIN and more when the launch has a staging area,
// else mode 1 for blocks of WARP_COPY_BYTES and more, else mode 2.  Modes 0
// and 2 copy blocks of at most TINY_BLOCK_BYTES one per thread.
template <class F>
static __device__ void multi_copy(int nb, int first, u64 avg_bytes, F f, int tid, int T, int mode = 0) {
    const bool staging = bulk_stage_bytes() >= 8192;
    if (staging && (mode == 3 || (mode == 0 && avg_bytes >= BULK_SEG_MIN))) {
        if (tid == 0) {
            BulkPipe bp;
            if (bp.begin()) {
                for (int k = 0; k < nb; k++) {
                    const void* s;
                    void* d;
                    u64 n;
                    if (!f((first + k) % nb, &s, &d, &n)) continue;
                    if ((((uintptr_t)s | (uintptr_t)d) & 15) == 0 && n >= 16 && !bp.push((char*)d, (const char*)s, n & ~(u64)15))
                        break;
                }
                bp.finish();
            }
        }
        const int warp = tid >> 5, lane = tid & 31, nw = T >> 5;
        for (int k = warp; k < nb; k += nw) {
            const void* s;
            void* d;
            u64 n;
            if (!f((first + k) % nb, &s, &d, &n)) continue;
            if ((((uintptr_t)s | (uintptr_t)d) & 15) == 0 && n >= 16) {
                const u64 n16 = n & ~(u64)15;
                if (n16 < n) warp_copy((char*)d + n16, (const char*)s + n16, n - n16, lane);
            } else {
                warp_copy(d, s, n, lane);
            }
        }
        bsync();
        return;
    }
    if ((mode == 0 || mode == 2) && avg_bytes <= TINY_BLOCK_BYTES) {
        // tiny blocks: one block per thread, all of them in flight at once
        // (a warp per block would wait one round trip per block)
        for (int k = tid; k < nb; k += T) {
            const void* s;
            void* d;
            u64 n;
            if (!f((first + k) % nb, &s, &d, &n)) continue;
            const char* sc = (const char*)s;
            char* dc = (char*)d;
            if ((((uintptr_t)sc | (uintptr_t)dc) & 15) == 0) {
                u64 i = 0;
                for (; i + 16 <= n; i += 16) *(uint4*)(dc + i) = __ldcg((const uint4*)(sc + i));
                for (; i < n; i++) dc[i] = __ldcg(sc + i);
            } else if ((((uintptr_t)sc | (uintptr_t)dc) & 7) == 0) {
                u64 i = 0;
                for (; i + 8 <= n; i += 8) *(u64*)(dc + i) = __ldcg((const u64*)(sc + i));
                for (; i < n; i++) dc[i] = __ldcg(sc + i);
            } else {
                for (u64 i = 0; i < n; i++) dc[i] = __ldcg(sc + i);
            }
        }
        bsync();
        return;
    }
    if (mode == 1 || mode == 3 || (mode == 0 && avg_bytes >= WARP_COPY_BYTES)) {
        for (int k = 0; k < nb; k++) {
            int q = (first + k) % nb;
            const void* s;
            void* d;
            u64 n;
            if (f(q, &s, &d, &n)) blk_copy(d, s, n, tid, T);
        }
    } else {
        const int warp = tid >> 5, lane = tid & 31, nw = T >> 5;
        for (int k = warp; k < nb; k += nw) {
            int q = (first + k) % nb;
            const void* s;
            void* d;
            u64 n;
            if (f(q, &s, &d, &n)) warp_copy(d, s, n, lane);
        }
    }
    bsync();
}

// ---------------------------------------------------------------- barrier
__device__ int coll_barrier(MPI_Comm_impl* c, int tid, int T) {
    const u64 seq = coll_begin(c, tid);
    const BlockCtx::CommView* cs = &bctx().cv;
    if (cs->P == 1) return MPI_SUCCESS;
    if (tid == 0) {
        __threadfence();
        st_release(&cs->arrive[cs->me], seq);
    }
    return wait_flags_ge(cs->arrive, cs->P, seq, cs->me, tid, T);
}

// ---------------------------------------------------------------- bcast
// Binomial tree (algo 2): with v = (rank - root) mod P, rank v copies from
// v with its lowest set bit cleared once that rank has its copy (its
// `arrive` flag), then raises its own; each rank returns once the ranks it
// feeds (v + 2^k below its lowest set bit) have copied from it (their
// `depart` flags).  log2(P) rounds, each reading a buffer at most log2(P)
// ranks read, against one round in which P - 1 ranks read the root's buffer.
static __device__ int bcast_tree(const CollArgs& a, u64 seq, int tid, int T) {
    const BlockCtx::CommView* cs = &bctx().cv;
    const int P = cs->P, me = cs->me, root = a.root;
    const int v = (me - root + P) % P;
    Pub p = {};
    p.sbuf = a.rbuf;
    if (v != 0) {
        const int pv = v & (v - 1);
        const int parent = (pv + root) % P;
        int rc = wait_one(cs->arrive, parent, seq, tid);
        if (rc) return rc;
        blk_copy(a.rbuf, ldcg(&cs->pub[parent].sbuf), a.count, tid, T);
        bsync();
        if (tid == 0) cs->pub[me] = p;
        raise_flag(cs->arrive, me, seq, tid);
        raise_flag(cs->depart, me, seq, tid);
    } else {
        if (tid == 0) cs->pub[me] = p;
        raise_flag(cs->arrive, me, seq, tid);
    }
    // the ranks this one feeds: v + 2^k for 2^k below v's lowest set bit (all k for the root)
    const int low = v ? (v & -v) : (1 << 30);
    int rc = MPI_SUCCESS;
    if (tid == 0) {
        for (int k = 1; k < low && v + k < P; k <<= 1) {
            rc = wait_ge(&cs->depart[(v + k + root) % P], seq);
            if (rc) break;
        }
    }
    return (int)bcast(rc, tid);
}

// a.rbuf = buffer, a.count = bytes.
__device__ int coll_bcast(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me, root = a.root;
    if (P == 1 || a.count == 0) return MPI_SUCCESS;
    if (a.algo == 2) return bcast_tree(a, seq, tid, T);
    if (me == root) {
        Pub p = {};
        p.sbuf = a.rbuf;
        publish(c, seq, p, tid);
        return wait_flags_ge(cs->depart, P, seq, me, tid, T);
    }
    int rc = wait_one(cs->arrive, root, seq, tid);
    if (rc) return rc;
    blk_copy(a.rbuf, ldcg(&cs->pub[root].sbuf), a.count, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- reduce
// a.sbuf (or MPI_IN_PLACE at the root), a.rbuf at the root, a.count elements
// of base type a.dtype (size a.rsize).
__device__ int coll_reduce(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me, root = a.root;
    const int es = a.rsize;
    const u64 n = a.count;
    const void* input = (a.sbuf == MPI_IN_PLACE && me == root) ? (const void*)a.rbuf : a.sbuf;
    if (P == 1) {
        if (input != a.rbuf) blk_copy(a.rbuf, input, n * es, tid, T);
        bsync();
        return MPI_SUCCESS;
    }
    Pub p = {};
    p.sbuf = input;
    p.rbuf = (me == root) ? a.rbuf : nullptr;
    publish(c, seq, p, tid);
    int rc;
    const bool root_only = (a.algo == 1) || (a.algo == 0 && n * es * (u64)P <= REDUCE_ROOT_ONLY_BYTES);
    if (root_only) {
        if (me == root) {
            rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
            if (rc) return rc;
            fold_range(a.opi, a.ufn, a.dtype, a.rsize, a.rbuf, cs->pub, P, 0, 0, n, tid, T);
            raise_flag(cs->depart, me, seq, tid);
            return MPI_SUCCESS;
        }
        return wait_one(cs->depart, root, seq, tid);
    }
    rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    const u64 per = seg_len(n, P, es);
    u64 lo = (u64)me * per;
    if (lo > n) lo = n;
    u64 hi = lo + per;
    if (hi > n) hi = n;
    char* out = (char*)ldcg(&cs->pub[root].rbuf) + lo * es;
    if (hi > lo) fold_range(a.opi, a.ufn, a.dtype, a.rsize, out, cs->pub, P, 0, lo, hi, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

// ---------------------------------------------------------------- allreduce
__device__ int coll_allreduce(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me;
    const int es = a.rsize;
    const u64 n = a.count;
    const bool in_place = a.sbuf == MPI_IN_PLACE;
    const void* input = in_place ? (const void*)a.rbuf : a.sbuf;
    if (P == 1) {
        if (input != a.rbuf) blk_copy(a.rbuf, input, n * es, tid, T);
        bsync();
        return MPI_SUCCESS;
    }
    Pub p = {};
    p.sbuf = input;
    p.rbuf = a.rbuf;
    publish(c, seq, p, tid);
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    const bool direct = (a.algo == 1) || (a.algo == 0 && n * es <= ALLREDUCE_DIRECT_BYTES);
    if (direct && !in_place) {
        // Every rank folds all inputs itself: one synchronisation round less.
        fold_range(a.opi, a.ufn, a.dtype, a.rsize, a.rbuf, cs->pub, P, 0, 0, n, tid, T);
        raise_flag(cs->depart, me, seq, tid);
        return wait_flags_ge(cs->depart, P, seq, me, tid, T);
    }
    const u64 per = seg_len(n, P, es);
    u64 lo = (u64)me * per;
    if (lo > n) lo = n;
    u64 hi = lo + per;
    if (hi > n) hi = n;
    // Pushing form: fold this rank's segment and write it into every rank's
    // receive buffer (traffic 2*P*n*s, one synchronisation round).
    if ((a.algo == 3 || a.algo == 0) && fold_range_push(a.opi, a.dtype, cs->pub, P, lo, hi, tid, T)) {
        raise_flag(cs->depart, me, seq, tid);
        return wait_flags_ge(cs->depart, P, seq, me, tid, T);
    }
    // Reduce-scatter into the owner's own receive buffer, then allgather by pull.
    if (hi > lo) fold_range(a.opi, a.ufn, a.dtype, a.rsize, (char*)a.rbuf + lo * es, cs->pub, P, 0, lo, hi, tid, T);
    raise_flag(cs->mid, me, seq, tid);
    rc = wait_flags_ge(cs->mid, P, seq, me, tid, T);
    if (rc) return rc;
    auto seg = [&](int q, const void** s, void** d, u64* nb) -> bool {
        if (q == me) return false;
        u64 l = (u64)q * per;
        if (l >= n) return false;
        u64 h = l + per;
        if (h > n) h = n;
        *s = (const char*)ldcg(&cs->pub[q].rbuf) + l * es;
        *d = (char*)a.rbuf + l * es;
        *nb = (h - l) * es;
        return true;
    };
    multi_copy(P, me + 1, per * es, seg, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

// Uniform or per-rank counts/displacements (elements).
static __device__ __forceinline__ u64 cnt_of(const int* arr, long long uni, int q) {
    return arr ? (u64)(long long)arr[q] : (u64)uni;
}
static __device__ __forceinline__ u64 dsp_of(const int* arr, long long uni, int q) {
    return arr ? (u64)(long long)arr[q] : (u64)uni * (u64)q;
}

// ---------------------------------------------------------------- gather(v)
// send: a.sbuf, a.a1 elements of a.ssize; root: a.rbuf, rcounts/rdispls (or a.a0 uniform).
__device__ int coll_gatherv(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me, root = a.root;
    Pub p = {};
    p.sbuf = a.sbuf;
    p.a0 = a.a1 * a.ssize;
    if (me != root) {
        publish(c, seq, p, tid);
        return wait_one(cs->depart, root, seq, tid);
    }
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    const int rs = a.rsize;
    u64 total = 0;
    for (int q = 0; q < P; q++) total += cnt_of(a.rcounts, a.a0, q);
    auto blk = [&](int q, const void** s, void** d, u64* nb) -> bool {
        if (q == me && a.sbuf == MPI_IN_PLACE) return false;
        u64 want = cnt_of(a.rcounts, a.a0, q) * rs;
        u64 have = q == me ? (u64)(a.a1 * a.ssize) : (u64)ldcg(&cs->pub[q].a0);
        *s = q == me ? a.sbuf : ldcg(&cs->pub[q].sbuf);
        *d = (char*)a.rbuf + dsp_of(a.rdispls, a.a0, q) * rs;
        *nb = want < have ? want : have;
        return true;
    };
    multi_copy(P, me, total * rs / (P ? P : 1), blk, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- scatter(v)
// root: a.sbuf with scounts/sdispls (or a.a1 uniform), a.ssize; everyone: a.rbuf, a.a0 elements of a.rsize.
__device__ int coll_scatterv(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me, root = a.root;
    const bool in_place = (me == root && a.rbuf == MPI_IN_PLACE);
    if (me == root) {
        Pub p = {};
        p.sbuf = a.sbuf;
        p.scounts = a.scounts;
        p.sdispls = a.sdispls;
        p.a0 = a.a1;
        p.a1 = a.ssize;
        publish(c, seq, p, tid);
        if (!in_place) {
            u64 n = cnt_of(a.scounts, a.a1, me) * a.ssize;
            u64 want = (u64)a.a0 * a.rsize;
            blk_copy(a.rbuf, (const char*)a.sbuf + dsp_of(a.sdispls, a.a1, me) * a.ssize,
                     n < want ? n : want, tid, T);
        }
        bsync();
        return wait_flags_ge(cs->depart, P, seq, me, tid, T);
    }
    int rc = wait_one(cs->arrive, root, seq, tid);
    if (rc) return rc;
    const Pub rp = load_pub(&cs->pub[root]);
    u64 n = cnt_of(rp.scounts, rp.a0, me) * (u64)rp.a1;
    u64 want = (u64)a.a0 * a.rsize;
    blk_copy(a.rbuf, (const char*)rp.sbuf + dsp_of(rp.sdispls, rp.a0, me) * (u64)rp.a1,
             n < want ? n : want, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- allgather(v)
// a.sbuf (or MPI_IN_PLACE), a.a1 elements of a.ssize; a.rbuf with rcounts/rdispls (or a.a0 uniform).
__device__ int coll_allgatherv(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me;
    const int rs = a.rsize;
    const bool in_place = a.sbuf == MPI_IN_PLACE;
    Pub p = {};
    if (in_place) {
        p.sbuf = (const char*)a.rbuf + dsp_of(a.rdispls, a.a0, me) * rs;
        p.a0 = cnt_of(a.rcounts, a.a0, me) * rs;
    } else {
        p.sbuf = a.sbuf;
        p.a0 = a.a1 * a.ssize;
    }
    publish(c, seq, p, tid);
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    u64 total = 0;
    for (int q = 0; q < P; q++) total += cnt_of(a.rcounts, a.a0, q);
    auto blk = [&](int q, const void** s, void** d, u64* nb) -> bool {
        if (q == me && in_place) return false;
        u64 want = cnt_of(a.rcounts, a.a0, q) * rs;
        u64 have = (u64)ldcg(&cs->pub[q].a0);
        *s = ldcg(&cs->pub[q].sbuf);
        *d = (char*)a.rbuf + dsp_of(a.rdispls, a.a0, q) * rs;
        *nb = want < have ? want : have;
        return true;
    };
    multi_copy(P, me, total * rs / P, blk, tid, T, a.algo);
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

// ---------------------------------------------------------------- alltoall(v)
// a.sbuf with scounts/sdispls (or a.a1 uniform) of a.ssize; a.rbuf with rcounts/rdispls
// (or a.a0 uniform) of a.rsize.
__device__ int coll_alltoallv(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me;
    const int rs = a.rsize;
    Pub p = {};
    p.sbuf = a.sbuf;
    p.scounts = a.scounts;
    p.sdispls = a.sdispls;
    p.a0 = a.a1;
    p.a1 = a.ssize;
    publish(c, seq, p, tid);
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    u64 total = 0;
    for (int q = 0; q < P; q++) total += cnt_of(a.rcounts, a.a0, q);
    auto blk = [&](int q, const void** s, void** d, u64* nb) -> bool {
        const Pub pq = load_pub(&cs->pub[q]);
        u64 have = cnt_of(pq.scounts, pq.a0, me) * (u64)pq.a1;
        u64 want = cnt_of(a.rcounts, a.a0, q) * rs;
        *s = (const char*)pq.sbuf + dsp_of(pq.sdispls, pq.a0, me) * (u64)pq.a1;
        *d = (char*)a.rbuf + dsp_of(a.rdispls, a.a0, q) * rs;
        *nb = want < have ? want : have;
        return *nb > 0;
    };
    multi_copy(P, me, total * rs / P, blk, tid, T, a.algo);
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

__device__ int coll_alltoall(const CollArgs& a, int tid, int T) { return coll_alltoallv(a, tid, T); }

// ---------------------------------------------------------------- reduce_scatter_block
// a.sbuf (P * a.count elements, or MPI_IN_PLACE: input in a.rbuf), a.rbuf (a.count elements).
__device__ int coll_reduce_scatter_block(const CollArgs& a, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me;
    const int es = a.rsize;
    const u64 n = a.count;
    if (a.sbuf == MPI_IN_PLACE) return GPUMPI_ERR_UNSUPPORTED;
    Pub p = {};
    p.sbuf = a.sbuf;
    publish(c, seq, p, tid);
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    fold_range(a.opi, a.ufn, a.dtype, a.rsize, a.rbuf, cs->pub, P, 0, (u64)me * n, (u64)me * n + n, tid, T);
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

// ---------------------------------------------------------------- scan / exscan
__device__ int coll_scan(const CollArgs& a, int exclusive, int tid, int T) {
    MPI_Comm_impl* c = a.comm;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(c, tid);
    const int P = cs->P, me = cs->me;
    const int es = a.rsize;
    const u64 n = a.count;
    if (a.sbuf == MPI_IN_PLACE) return GPUMPI_ERR_UNSUPPORTED;
    Pub p = {};
    p.sbuf = a.sbuf;
    publish(c, seq, p, tid);
    const int nin = exclusive ? me : me + 1;
    int rc = wait_flags_ge(cs->arrive, nin, seq, me, tid, T);
    if (rc) return rc;
    if (nin > 0) fold_range(a.opi, a.ufn, a.dtype, a.rsize, a.rbuf, cs->pub, nin, 0, 0, n, tid, T);
    (void)es;
    raise_flag(cs->depart, me, seq, tid);
    return wait_flags_ge(cs->depart, P, seq, me, tid, T);
}

// ---------------------------------------------------------------- launch-ordered forms
// A host plan whose calls touch disjoint memory (the plan checks every pair of
// calls on the host) needs no arrive and no depart round: every input was
// written before the launch started (stream order), no call of the launch
// writes what another reads, and the end of the launch orders every result
// before whatever follows it on the stream.  These forms therefore read the
// peers' buffers from a table the plan built on the host (`pub`, one entry per
// rank) and synchronise nothing but their own rank block, so a rank never waits
// for a slower peer.  The one exception is the reduce-scatter + allgather
// Allreduce: its allgather reads what the reduce-scatter wrote in the same
// launch, so it keeps its middle flag round.  The arithmetic and the fold
// order are those of the synchronised forms above.

// Bcast: a.rbuf of every rank receives a.count bytes of the root's.
__device__ int coll_lo_bcast(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T) {
    if (P > 1 && me != a.root && a.count) blk_copy(a.rbuf, ldcg(&pub[a.root].rbuf), a.count, tid, T);
    bsync();
    return MPI_SUCCESS;
}

// Reduce to a.root (a.sbuf == a.rbuf at the root works in place).
__device__ int coll_lo_reduce(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T) {
    const int es = a.rsize;
    const u64 n = a.count;
    if (P == 1) {
        if (a.sbuf != a.rbuf) blk_copy(a.rbuf, a.sbuf, n * es, tid, T);
        bsync();
        return MPI_SUCCESS;
    }
    const bool root_only = (a.algo == 1) || (a.algo == 0 && n * es * (u64)P <= REDUCE_ROOT_ONLY_BYTES);
    if (root_only) {
        if (me == a.root) fold_range(a.opi, a.ufn, a.dtype, es, a.rbuf, pub, P, 0, 0, n, tid, T);
        bsync();
        return MPI_SUCCESS;
    }
    const u64 per = seg_len(n, P, es);
    u64 lo = (u64)me * per;
    if (lo > n) lo = n;
    u64 hi = lo + per;
    if (hi > n) hi = n;
    char* out = (char*)ldcg(&pub[a.root].rbuf) + lo * es;
    if (hi > lo) fold_range(a.opi, a.ufn, a.dtype, es, out, pub, P, 0, lo, hi, tid, T);
    bsync();
    return MPI_SUCCESS;
}

// Allreduce (a.sbuf == a.rbuf works in place).
__device__ int coll_lo_allreduce(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T) {
    const int es = a.rsize;
    const u64 n = a.count;
    const bool in_place = a.sbuf == a.rbuf;
    if (P == 1) {
        if (!in_place) blk_copy(a.rbuf, a.sbuf, n * es, tid, T);
        bsync();
        return MPI_SUCCESS;
    }
    const bool direct = (a.algo == 1) || (a.algo == 0 && n * es <= ALLREDUCE_DIRECT_BYTES);
    if (direct && !in_place) {
        // every rank folds every input into its own receive buffer
        fold_range(a.opi, a.ufn, a.dtype, es, a.rbuf, pub, P, 0, 0, n, tid, T);
        return MPI_SUCCESS;
    }
    const u64 per = seg_len(n, P, es);
    u64 lo = (u64)me * per;
    if (lo > n) lo = n;
    u64 hi = lo + per;
    if (hi > n) hi = n;
    if (a.algo != 2 && fold_range_push(a.opi, a.dtype, pub, P, lo, hi, tid, T)) return MPI_SUCCESS;
    // reduce-scatter into the owner's receive buffer, one flag round, allgather
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(a.comm, tid);
    if (hi > lo) fold_range(a.opi, a.ufn, a.dtype, es, (char*)a.rbuf + lo * es, pub, P, 0, lo, hi, tid, T);
    raise_flag(cs->mid, me, seq, tid);
    const int rc = wait_flags_ge(cs->mid, P, seq, me, tid, T);
    if (rc) return rc;
    auto seg = [&](int q, const void** s, void** d, u64* nb) -> bool {
        if (q == me) return false;
        u64 l = (u64)q * per;
        if (l >= n) return false;
        u64 h = l + per;
        if (h > n) h = n;
        *s = (const char*)ldcg(&pub[q].rbuf) + l * es;
        *d = (char*)a.rbuf + l * es;
        *nb = (h - l) * es;
        return true;
    };
    multi_copy(P, me + 1, per * es, seg, tid, T);
    return MPI_SUCCESS;
}

// Alltoall / Allgather with a uniform block of a.count elements of a.rsize
// bytes: block q of this rank's a.rbuf comes from rank q (Alltoall: its block
// for this rank; Allgather: its whole send buffer).
// Schedule 4 (and the choice for blocks of TINY_BLOCK_BYTES to BULK_SEG_MIN
// when the buffers are 16-byte aligned): the 16-byte vectors of all P blocks
// form one index space spread over every thread of the rank block, 8 loads in
// flight per thread, the source bases in a shared-memory table.  Per-warp or
// per-block copies of such blocks leave most threads idle (a 512-byte block
// is one vector per lane of one warp) and wait one round trip per block.
static __device__ bool alltoall_flat(const CollArgs& a, const Pub* pub, int P, int me, int gather, u64 b, int tid,
                                     int T) {
    extern __shared__ __align__(16) char gm_dsmem[];
    if (b % 16 != 0 || bulk_stage_bytes() < (u32)P * sizeof(char*) || ((uintptr_t)a.rbuf & 15)) return false;
    const char** tab = reinterpret_cast<const char**>(gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES);
    int bad = 0;
    for (int q = tid; q < P; q += T) {
        tab[q] = (const char*)ldcg(&pub[q].sbuf) + (gather ? 0 : (u64)me * b);
        bad |= ((uintptr_t)tab[q] & 15) != 0;
    }
    if (bar_or(bad, T)) return false;   // the same answer on every rank: all see the same table
    const u64 nv = b / 16, total = (u64)P * nv;
    uint4* out = reinterpret_cast<uint4*>(a.rbuf);
    constexpr int U = 8;
    // vector k = q * nv + v of the output comes from vector v of peer q's block;
    // (q, v) advance by the quotient and remainder of the stride instead of a
    // 64-bit division per vector
    const u64 sq = (u64)T / nv, sv = (u64)T % nv;
    const u64 bq = (u64)U * T / nv, bv = (u64)U * T % nv;
    u64 q0 = (u64)tid / nv, v0 = (u64)tid % nv;
    for (u64 k0 = (u64)tid; k0 < total; k0 += (u64)U * T) {
        uint4 v[U];
        u64 q = q0, w = v0;
#pragma unroll
        for (int u = 0; u < U; u++) {
            if (q < (u64)P) v[u] = __ldcg(reinterpret_cast<const uint4*>(tab[q]) + w);
            q += sq;
            w += sv;
            if (w >= nv) {
                w -= nv;
                q++;
            }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const u64 k = k0 + (u64)u * T;
            if (k < total) out[k] = v[u];
        }
        q0 += bq;
        v0 += bv;
        if (v0 >= nv) {
            v0 -= nv;
            q0++;
        }
    }
    bsync();
    return true;
}

__device__ int coll_lo_alltoall(const CollArgs& a, const Pub* pub, int P, int me, int gather, int tid, int T) {
    const u64 b = a.count * (u64)a.rsize;
    if (b == 0) {
        bsync();
        return MPI_SUCCESS;
    }
    const bool flat = a.algo == 4 || (a.algo == 0 && b > TINY_BLOCK_BYTES && b < BULK_SEG_MIN);
    if (flat && alltoall_flat(a, pub, P, me, gather, b, tid, T)) return MPI_SUCCESS;
    auto blk = [&](int q, const void** s, void** d, u64* nb) -> bool {
        *s = (const char*)ldcg(&pub[q].sbuf) + (gather ? 0 : (u64)me * b);
        *d = (char*)a.rbuf + (u64)q * b;
        *nb = b;
        return true;
    };
    multi_copy(P, me, b, blk, tid, T, a.algo == 4 ? 0 : a.algo);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- communicator creation
static __device__ CommShared* arena_comm(Job* j, int size) {
    u64 bytes = sizeof(CommShared) + (u64)size * (sizeof(int) + sizeof(Pub) + 3 * sizeof(u64)) + 256;
    bytes = (bytes + 255) & ~255ull;
    u64 off = atomicAdd(j->arena_off, bytes);
    if (off + bytes > j->arena_bytes) return nullptr;
    char* base = j->arena + off;
    CommShared* cs = (CommShared*)base;
    char* q = base + ((sizeof(CommShared) + 127) & ~127ull);
    cs->pub = (Pub*)q;
    q += (u64)size * sizeof(Pub);
    cs->arrive = (u64*)q;
    q += (u64)size * sizeof(u64);
    cs->mid = (u64*)q;
    q += (u64)size * sizeof(u64);
    cs->depart = (u64*)q;
    q += (u64)size * sizeof(u64);
    cs->members = (int*)q;
    cs->size = size;
    return cs;
}

// Split `parent` by (color, key); new ranks ordered by (key, parent rank) as in
// gpu_libs/gpu_mpi/communicator.cu:154-199.  color < 0 (MPI_UNDEFINED) yields
// no communicator.  Used for Comm_split, Comm_dup and Comm_create.
__device__ int comm_split_block(MPI_Comm_impl* parent, int color, int key, MPI_Comm_impl** out,
                                int tid, int T) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    const BlockCtx::CommView* cs = &bctx().cv;
    const u64 seq = coll_begin(parent, tid);
    const int P = cs->P, me = cs->me;
    Pub p = {};
    p.a0 = color;
    p.a1 = key;
    publish(parent, seq, p, tid);
    int rc = wait_flags_ge(cs->arrive, P, seq, me, tid, T);
    if (rc) return rc;
    // Count members of my color that order before me, the color size, and the
    // color's first member (who allocates the shared state).
    __shared__ unsigned int s_before, s_size;
    __shared__ unsigned long long s_lead;
    if (tid == 0) {
        s_before = 0;
        s_size = 0;
        s_lead = ~0ull;
    }
    bsync();
    if (color >= 0) {
        const unsigned long long mine = ((unsigned long long)((long long)key + 0x80000000ll) << 32) | (unsigned)me;
        for (int q = tid; q < P; q += T) {
            if ((int)ldcg(&cs->pub[q].a0) != color) continue;
            const long long kq = ldcg(&cs->pub[q].a1);
            const unsigned long long vq = ((unsigned long long)(kq + 0x80000000ll) << 32) | (unsigned)q;
            atomicAdd(&s_size, 1u);
            if (vq < mine) atomicAdd(&s_before, 1u);
            atomicMin(&s_lead, vq);
        }
    }
    bsync();
    const int newrank = (int)s_before, newsize = (int)s_size;
    const int leader = (int)(s_lead & 0xffffffffu);
    bsync();
    if (tid == 0 && color >= 0 && newrank == 0) {
        CommShared* ncs = arena_comm(j, newsize);
        if (ncs) ncs->ctx = 3 + atomicAdd(&j->status[5], 1);
        cs->pub[me].rbuf = ncs;
    }
    raise_flag(cs->mid, me, seq, tid);
    MPI_Comm_impl* h = nullptr;
    if (color >= 0) {
        rc = wait_one(cs->mid, leader, seq, tid);
        if (rc) return rc;
        CommShared* ncs = (CommShared*)ldcg(&cs->pub[leader].rbuf);
        if (tid == 0 && ncs) {
            ncs->members[newrank] = comm_world_rank(parent, me);
            RankPriv* pr = b.priv;
            for (int i = 2; i < MAX_COMMS; i++) {
                if (pr->comms[i].kind == 0) {
                    h = &pr->comms[i];
                    break;
                }
            }
            if (h) {
                h->kind = 1;
                h->ctx = ncs->ctx;
                h->size = newsize;
                h->rank = newrank;
                h->refcnt = 1;
                h->cs = ncs;
                h->seq = 0;
            }
        }
        if (tid == 0 && !ncs) rc = MPI_ERR_NO_MEM;
        if (tid == 0 && ncs && !h) rc = MPI_ERR_INTERN;
    }
    raise_flag(cs->depart, me, seq, tid);
    int rc2 = wait_flags_ge(cs->depart, P, seq, me, tid, T);
    if (tid == 0) *out = h;
    rc = (int)bcast(rc, tid);
    return rc ? rc : rc2;
}

}  // namespace gm
