// Point-to-point engine: per-receiver HBM mailboxes with warp-ballot matching,
// eager delivery into mailbox slots for small messages and receiver-pull
// rendezvous for large ones.  All functions here are block-cooperative: every
// thread of the rank block calls them with its thread index.
//
// Ownership rule: thread 0 (the rank's leader) is the only thread that reads
// or writes rank-private state (request objects, the posted-receive and
// deferred-send lists).  It hands the block what it needs -- match keys,
// copy source/destination/length -- through shared memory (bctx().x), so the
// other threads never load memory the leader wrote.  Data written by other
// ranks (mailbox headers, payloads) is read through L2 (ld.global.cg) after
// an acquire load of the mailbox's ready mask.
//
// Semantics follow the reference transport (gpu_libs/gpu_libc/cuda_mpi.cu:
// 120-471: match-or-enqueue, progress of all pending operations in order)
// with its defects corrected:
//  * a send completes only once its bytes are in the mailbox (eager) or in
//    the receiver's buffer (rendezvous), never by lending the sender's buffer
//    (cuda_mpi.cu:176-212);
//  * wildcard source/tag match arrived messages as well as posted ones
//    (cuda_mpi.cu:300-304);
//  * messages between one sender and one receiver on one communicator match
//    in send order: the arrival stamp is taken after the slot is claimed, and a
//    sender publishes its messages one after the other, so the lowest matching
//    stamp is always the oldest message of that sender;
//  * every wait is bounded and returns an error code instead of spinning forever.
#include "rt.cuh"
#include "p2p_small.cuh"

namespace gm {

static __device__ __forceinline__ char* eager_slot(Job* j, int world_rank, int slot) {
    return j->eager + ((u64)world_rank * MB_SLOTS + slot) * j->eager_bytes;
}

// Thread 0: claim a free slot in the destination's mailbox and fill its header.
// Returns the slot, or -1 when the mailbox is full.
static __device__ int claim_and_fill(Job* j, MPI_Request_impl* r) {
    Mailbox* mb = mbox_of(r->peer_world);
    u64 used = mb_ld(&mb->used);
    int s;
    for (;;) {
        u64 freeb = ~used;
        if (freeb == 0) return -1;
        s = __ffsll((long long)freeb) - 1;
        u64 bit = 1ull << s;
        // acquire: a slot freed by the receiver's release of `used` is claimed
        // only after the receiver's clear of its ready bit
        u64 old = mb_atom_or_acquire(&mb->used, bit);
        if (!(old & bit)) break;
        used |= old | bit;   // old holds the bit's 32-bit half only
    }
    u64 stamp = mb_atom_add(&mb->stamp, 1ull);
    MsgHdr& h = mb->hdr[s];
    const bool eager = r->bytes <= j->eager_bytes;
    h.ctx = r->ctx;
    h.src = r->src_rank;
    h.tag = r->tag;
    h.kind = eager ? 0 : 1;
    h.bytes = r->bytes;
    h.stamp = stamp;
    h.rdv_src = eager ? nullptr : r->buf;
    h.rdv_done = eager ? nullptr : (u32*)&r->done;
    if (eager && r->bytes <= INLINE_BYTES && r->bytes) {
        // the payload travels in the header
        unsigned char tmp[INLINE_BYTES];
        for (u64 i = 0; i < r->bytes; i++) tmp[i] = ((const unsigned char*)r->buf)[i];
        for (u64 i = r->bytes; i < INLINE_BYTES; i++) tmp[i] = 0;
        u64 w[2];
        memcpy(w, tmp, INLINE_BYTES);
        h.inl[0] = w[0];
        h.inl[1] = w[1];
    }
    return s;
}

// Thread 0: describe the eager copy of request r into `slot` in bctx().x.
static __device__ void stage_delivery(MPI_Request_impl* r, int slot) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    const bool eager = r->bytes <= j->eager_bytes;
    b.x.slot = slot;
    b.x.src = r->buf;
    b.x.dst = slot >= 0 ? eager_slot(j, r->peer_world, slot) : nullptr;
    b.x.bytes = (slot >= 0 && eager && r->bytes > INLINE_BYTES) ? r->bytes : 0;
    b.x.peer = r->peer_world;
    b.x.a = eager;
}

// All threads: copy the staged eager payload, then thread 0 publishes the slot.
static __device__ void deliver_staged(MPI_Request_impl* r, int tid, int T) {
    BlockCtx& b = bctx();
    const void* src = b.x.src;
    void* dst = b.x.dst;
    const u64 n = b.x.bytes;
    const int slot = b.x.slot, peer = b.x.peer, eager = b.x.a;
    if (n) blk_copy(dst, src, n, tid, T);
    bsync();
    if (tid == 0) {
        r->state = eager ? RS_DONE : RS_WAIT_RDV;
        // release: the header and the payload copied by the block (ordered by
        // the barrier above) become visible before the ready bit
        mb_red_or_release(&mbox_of(peer)->ready, 1ull << slot);
    }
}

static __device__ void list_append(RankPriv* p, int* head, int* tail, int idx) {
    p->reqs[idx].next = -1;
    if (*tail >= 0) p->reqs[*tail].next = idx;
    else *head = idx;
    *tail = idx;
}

__device__ int p2p_send_start(MPI_Request_impl* r, int tid, int T) {
    BlockCtx& b = bctx();
    bsync();
    if (tid == 0) {
        RankPriv* p = b.priv;
        int slot = -1;
        r->done = 0;
        if (p->defer_head < 0) slot = claim_and_fill(b.job, r);
        if (slot < 0) {
            r->state = RS_DEFERRED;
            list_append(p, &p->defer_head, &p->defer_tail, r->index);
        }
        stage_delivery(r, slot);
    }
    bsync();
    if (b.x.slot >= 0) deliver_staged(r, tid, T);
    return MPI_SUCCESS;
}

// Warp 0 finds the earliest ready message matching the keys in bctx().x
// (ctx/peer/tag) among the slots of `ready`; the result is valid in lane 0.
static __device__ int warp_match(u64 ready, int tid) {
    BlockCtx& b = bctx();
    int best = -1;
    if (tid < 32) {
        const int ctx = b.x.ctx, src = b.x.peer, tag = b.x.tag;
        Mailbox* mb = mbox_of(b.rank);
        u64 best_stamp = ~0ull;
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int s = tid + 32 * k;
            if ((ready >> s) & 1ull) {
                const MsgHdr* h = &mb->hdr[s];
                const int4 h0 = mb_ld4(h);   // ctx, src, tag, kind
                const int hctx = h0.x, hsrc = h0.y, htag = h0.z;
                if (hctx == ctx && (src == MPI_ANY_SOURCE || hsrc == src) &&
                    (tag == MPI_ANY_TAG || htag == tag)) {
                    const u64 st = mb_ld(&h->stamp);
                    if (st < best_stamp) {
                        best_stamp = st;
                        best = s;
                    }
                }
            }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const u64 os = __shfl_xor_sync(0xffffffffu, best_stamp, off);
            const int ob = __shfl_xor_sync(0xffffffffu, best, off);
            if (os < best_stamp) {
                best_stamp = os;
                best = ob;
            }
        }
    }
    return best;
}

// One pass over posted receives, in posting order, against one snapshot of the
// ready mask.  Thread 0 walks the list; for each receive the block matches
// and, on a hit, copies.  Every message of the snapshot goes to the earliest
// posted receive it matches, which is MPI's matching rule.
static __device__ int progress_recvs(int tid, int T) {
    BlockCtx& b = bctx();
    RankPriv* p = b.priv;
    Mailbox* mb = mbox_of(b.rank);
    int did = 0;
    // thread-0 walk state
    int cur = -1, prev = -1;
    u64 ready = 0;
    if (tid == 0) {
        ready = mb_ld_acquire(&mb->ready);
        cur = ready ? p->recv_head : -1;
    }
    for (;;) {
        bsync();
        if (tid == 0) {
            b.x.a = cur >= 0;
            if (cur >= 0) {
                const MPI_Request_impl* r = &p->reqs[cur];
                b.x.ctx = r->ctx;
                b.x.peer = r->peer;
                b.x.tag = r->tag;
                b.bval = ready;
            }
        }
        bsync();
        if (!b.x.a) break;
        const int best = warp_match(b.bval, tid);
        bsync();
        if (tid == 0) {
            b.x.slot = best;
            if (best >= 0) {
                const MPI_Request_impl* r = &p->reqs[cur];
                const MsgHdr* h = &mb->hdr[best];
                const u64 bytes = mb_ld(&h->bytes);
                const int kind = mb_ld_int(&h->kind);
                const u64 n = bytes < r->bytes ? bytes : r->bytes;
                b.x.dst = r->buf;
                if (kind == 0 && bytes <= INLINE_BYTES) {
                    // the payload is in the header: the leader copies it
                    const ulonglong2 w = mb_ld2(&h->inl);
                    const unsigned char* pc = (const unsigned char*)&w;
                    for (u64 i = 0; i < n; i++) ((unsigned char*)r->buf)[i] = pc[i];
                    b.x.src = nullptr;
                    b.x.bytes = 0;
                } else {
                    b.x.src = kind == 0 ? (const void*)eager_slot(b.job, b.rank, best) : (const void*)mb_ld((const u64*)&h->rdv_src);
                    b.x.bytes = n;
                }
            }
        }
        bsync();
        const int slot = b.x.slot;
        if (slot >= 0) {
            blk_copy(b.x.dst, b.x.src, b.x.bytes, tid, T);
            bsync();
            if (tid == 0) {
                MPI_Request_impl* r = &p->reqs[cur];
                const MsgHdr* h = &mb->hdr[slot];
                const u64 bytes = mb_ld(&h->bytes);
                const int4 h0 = mb_ld4(h);   // ctx, src, tag, kind
                r->st_source = h0.y;
                r->st_tag = h0.z;
                r->st_bytes = bytes < r->bytes ? bytes : r->bytes;
                r->st_err = bytes > r->bytes ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
                u32* done = h0.w == 1 ? (u32*)mb_ld((const u64*)&h->rdv_done) : nullptr;
                mb_red_and_relaxed(&mb->ready, ~(1ull << slot));
                if (done) {
                    __threadfence();
                    st_release32(done, 1u);
                }
                // release: the ready clear and the reads of the slot come before
                // the slot can be claimed again
                mb_red_and_release(&mb->used, ~(1ull << slot));
                r->state = RS_DONE;
                const int nxt = r->next;
                if (prev >= 0) p->reqs[prev].next = nxt;
                else p->recv_head = nxt;
                if (p->recv_tail == cur) p->recv_tail = prev;
                cur = nxt;
                // The pass keeps its snapshot: a message that arrived after it
                // was taken must go to the earliest matching receive, which
                // this pass may already have walked past; the next pass starts
                // again at the head of the list.
                ready &= ~(1ull << slot);
                if (!ready) cur = -1;
            }
            did = 1;
        } else if (tid == 0) {
            prev = cur;
            cur = p->reqs[cur].next;
        }
    }
    return did;
}

// Retry sends that found the destination mailbox full, oldest first.
static __device__ int progress_deferred(int tid, int T) {
    BlockCtx& b = bctx();
    RankPriv* p = b.priv;
    int did = 0;
    for (;;) {
        bsync();
        if (tid == 0) {
            int slot = -1;
            const int h = p->defer_head;
            b.x.c = h;
            if (h >= 0) {
                MPI_Request_impl* r = &p->reqs[h];
                slot = claim_and_fill(b.job, r);
                if (slot >= 0) {
                    p->defer_head = r->next;
                    if (p->defer_head < 0) p->defer_tail = -1;
                }
                stage_delivery(r, slot);
            } else {
                b.x.slot = -1;
            }
        }
        bsync();
        if (b.x.slot < 0) break;
        deliver_staged(&p->reqs[b.x.c], tid, T);
        did = 1;
    }
    return did;
}

__device__ int p2p_progress(int tid, int T, int* did_work) {
    int d1 = progress_deferred(tid, T);
    int d2 = progress_recvs(tid, T);
    if (did_work) *did_work = d1 | d2;
    return MPI_SUCCESS;
}

__device__ int p2p_recv_post(MPI_Request_impl* r, int tid, int T) {
    BlockCtx& b = bctx();
    if (tid == 0) {
        RankPriv* p = b.priv;
        r->state = RS_POSTED;
        list_append(p, &p->recv_head, &p->recv_tail, r->index);
    }
    progress_recvs(tid, T);
    return MPI_SUCCESS;
}

static __device__ __forceinline__ int req_is_done(MPI_Request_impl* r) {
    if (r->state == RS_DONE) return 1;
    if (r->state == RS_WAIT_RDV && ld_acquire32((const u32*)&r->done)) {
        r->state = RS_DONE;
        return 1;
    }
    return 0;
}

// Thread 0: abort / timeout check of a wait loop.  Returns an error code or 0.
static __device__ int wait_check(u64 t0, int did, unsigned* ns, const char* what) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    if (job_aborted(j)) return fail_code(j);
    if (gtime() - t0 > j->timeout_ns) {
        job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, what);
        return GPUMPI_ERR_TIMEOUT;
    }
    if (!did) {
        __nanosleep(*ns);
        if (*ns < 256) *ns <<= 1;
    } else {
        *ns = 32;
    }
    return 0;
}

// Progress until r completes (blocking) or for one pass (non-blocking).
// Non-blocking calls report completion in call.a[1].
__device__ int p2p_wait(MPI_Request_impl* r, int tid, int T, int blocking) {
    BlockCtx& b = bctx();
    u64 t0 = 0;
    unsigned ns = 32;
    if (tid == 0) t0 = gtime();
    for (int iter = 0;; iter++) {
        int done = (int)bcast(tid == 0 ? req_is_done(r) : 0, tid);
        if (done || (!blocking && iter > 0)) {
            if (!blocking && tid == 0) b.call.a[1] = (u64)done;
            return MPI_SUCCESS;
        }
        int did = 0;
        p2p_progress(tid, T, &did);
        int code = 0;
        if (tid == 0 && blocking) code = wait_check(t0, did, &ns, "point-to-point wait timed out");
        code = (int)bcast(code, tid);
        if (code) return code;
    }
}

// Look for a matching arrived message without receiving it.  Thread 0 (the
// leader) writes the status, so it may live in the leader's local memory.
__device__ int p2p_probe(int source, int tag, int ctx, int blocking, MPI_Status* st, int tid,
                         int T) {
    BlockCtx& b = bctx();
    Mailbox* mb = mbox_of(b.rank);
    u64 t0 = 0;
    unsigned ns = 32;
    if (tid == 0) t0 = gtime();
    for (;;) {
        int did = progress_deferred(tid, T);
        bsync();
        if (tid == 0) {
            b.bval = mb_ld_acquire(&mb->ready);
            b.x.ctx = ctx;
            b.x.peer = source;
            b.x.tag = tag;
        }
        bsync();
        const int best = b.bval ? warp_match(b.bval, tid) : -1;
        int found = 0;
        if (tid == 0 && best >= 0) {
            const MsgHdr* h = &mb->hdr[best];
            if (st) {
                const u64 hb = mb_ld(&h->bytes);
                const int4 h0 = mb_ld4(h);
                st->MPI_SOURCE = h0.y;
                st->MPI_TAG = h0.z;
                st->MPI_ERROR = MPI_SUCCESS;
                st->gpumpi_count_lo = (int)(hb & 0xffffffffu);
                st->gpumpi_count_hi = (int)(hb >> 32);
            }
            found = 1;
        }
        found = (int)bcast(found, tid);
        if (found || !blocking) {
            if (tid == 0) b.call.a[1] = (u64)found;
            return MPI_SUCCESS;
        }
        int code = 0;
        if (tid == 0) code = wait_check(t0, did, &ns, "probe timed out");
        code = (int)bcast(code, tid);
        if (code) return code;
    }
}

// ---------------------------------------------------------------- leader-only small messages
// Small eager messages need no block: the leader claims the slot, copies the
// payload and publishes it (send), or finds the oldest matching message,
// copies it out and frees the slot (blocking receive), without waking the
// helper threads.  It reads and writes the user's buffer itself, so a buffer in
// its local memory needs no staging.  The receive path is taken only when no
// receive is posted and no send is deferred, so message order and matching
// are the same as on the block path; anything else (a rendezvous message, a
// full mailbox) falls back to the block path before touching any state.

// One thread copies 16-byte vectors, 8 loads in flight before their stores (a
// load-store-load chain would wait a memory round trip per vector, as the
// compiler cannot move a load above a store that may alias it).  `cg`: the
// source is read through L2 (data another SM wrote).
template <bool cg>
static __device__ __forceinline__ void copy_vec16(uint4* d, const uint4* s, u64 nv) {
    u64 i = 0;
    for (; i + 8 <= nv; i += 8) {
        uint4 v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = cg ? __ldcg(s + i + k) : s[i + k];
#pragma unroll
        for (int k = 0; k < 8; k++) d[i + k] = v[k];
    }
    for (; i < nv; i++) d[i] = cg ? __ldcg(s + i) : s[i];
}

static __device__ void leader_copy(void* dst, const void* src, u64 n) {
    char* d = (char*)dst;
    const char* s = (const char*)src;
    if ((((uintptr_t)d | (uintptr_t)s) & 15) == 0) {
        const u64 nv = n >> 4;
        copy_vec16<false>((uint4*)d, (const uint4*)s, nv);
        for (u64 i = nv << 4; i < n; i++) d[i] = s[i];
    } else if ((((uintptr_t)d | (uintptr_t)s) & 7) == 0) {
        const u64 nv = n >> 3;
        for (u64 i = 0; i < nv; i++) ((u64*)d)[i] = ((const u64*)s)[i];
        for (u64 i = nv << 3; i < n; i++) d[i] = s[i];
    } else {
        for (u64 i = 0; i < n; i++) d[i] = s[i];
    }
}

// Leader: send r (r->buf may be local memory) without the block.  False: use the block path.
static __device__ int leader_bulk_copy(char* dst, const char* src, u64 n);
static __device__ bool leader_bulk_ok(const void* p, u64 n);

__device__ bool p2p_send_fast(MPI_Request_impl* r) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    // above FAST_MSG_BYTES only through the bulk engine (global, aligned buffer)
    const bool bulk = r->bytes > FAST_MSG_BYTES && leader_bulk_ok(r->buf, r->bytes);
    if ((r->bytes > FAST_MSG_BYTES && !bulk) || r->bytes > j->eager_bytes || b.priv->defer_head >= 0)
        return false;
    r->done = 0;
    const int slot = claim_and_fill(j, r);
    if (slot < 0) return false;
    char* dst = eager_slot(j, r->peer_world, slot);
    if (r->bytes <= INLINE_BYTES) {
        // claim_and_fill put the payload into the header
    } else if (bulk) {
        const u64 n16 = r->bytes & ~(u64)15;
        const int rc = leader_bulk_copy(dst, (const char*)r->buf, n16);
        if (rc) {   // the job has failed; nothing is published
            r->st_err = rc;
            r->state = RS_DONE;
            return true;
        }
        for (u64 i = n16; i < r->bytes; i++) dst[i] = ((const char*)r->buf)[i];
    } else if (r->bytes) {
        leader_copy(dst, r->buf, r->bytes);
    }
    mb_red_or_release(&mbox_of(r->peer_world)->ready, 1ull << slot);
    r->state = RS_DONE;
    return true;
}

// Leader: nonblocking rendezvous send from a global buffer while nothing is
// posted on the block path: the header points the receiver at r->buf and at
// r->done; the request then waits for the receiver's pull (rdv_wait_leader).
__device__ bool p2p_send_rdv_fast(MPI_Request_impl* r) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    if (r->bytes <= j->eager_bytes || !b.p2p_quiet || !is_global(r->buf)) return false;
    r->done = 0;
    const int slot = claim_and_fill(j, r);   // rendezvous header: rdv_src = r->buf, rdv_done = &r->done
    if (slot < 0) return false;
    mb_red_or_release(&mbox_of(r->peer_world)->ready, 1ull << slot);
    r->state = RS_WAIT_RDV;
    return true;
}

// Leader: wait until the receiver of rendezvous send r has pulled it, while
// progressing this rank's lazy receives (the receiver may be waiting for a
// rendezvous message of its own from this rank).  Returns 0 with r done, or 0
// with r still waiting when the block path must take over, or an error code.
__device__ int rdv_wait_leader(MPI_Request_impl* r) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    const u64 t0 = gtime();
    unsigned ns = 32;
    for (;;) {
        if (ld_acquire32((const u32*)&r->done)) {
            r->state = RS_DONE;
            return MPI_SUCCESS;
        }
        const int rc = lazy_progress();
        if (rc) return rc;
        if (!b.p2p_quiet) return MPI_SUCCESS;   // block path receives posted: wait there
        mb_release_taken();
        if (ld_relaxed_int(&j->status[0]) != 0) return fail_code(j);
        if (gtime() - t0 > b.timeout_ns) {
            job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
    }
}

// The leader alone copies n bytes (a multiple of 16) between 16-byte aligned
// global buffers through the bulk engine: one load and one store round trip,
// whatever n.  Returns 0 or an error code (the job has then failed).
static __device__ int leader_bulk_copy(char* dst, const char* src, u64 n) {
    BulkPipe bp;
    if (!bp.begin()) return MPI_ERR_INTERN;   // not reached: leader_bulk_ok checked the area
    bp.push(dst, src, n);
    return bp.finish();
}

static __device__ bool leader_bulk_ok(const void* p, u64 n) {
    return n >= SMALL_BULK_MIN && ((uintptr_t)p & 15) == 0 && is_global(p) && !bctx().bulk_broken &&
           bulk_stage_bytes() >= 8192;
}

// Leader: blocking rendezvous send without a request object.
// The header points the receiver at the user's (global) buffer and at the
// rank's completion word; the call returns once the receiver has copied the
// data and set that word.  Returns 0 (before publishing) when buf is not in
// global memory or the mailbox is full.
__device__ int p2p_send_rdv_small(const void* buf, u64 bytes, int dest_job, int ctx, int me, int tag, int* rc) {
    BlockCtx& b = bctx();
    if (!is_global(buf)) return 0;
    Mailbox* mb = mbox_of(dest_job);
    const u64 stamp = mb_atom_add(&mb->stamp, 1ull);
    u32* done = &b.priv->rdv_done_small;
    *done = 0u;
    const int s = claim_slot_small(mb);
    if (s < 0) return 0;
    MsgHdr* h = &mb->hdr[s];
    *(int4*)h = make_int4(ctx, me, tag, 1);   // kind = rendezvous
    *(ulonglong2*)&h->bytes = make_ulonglong2(bytes, stamp);
    *(ulonglong2*)&h->rdv_src = make_ulonglong2((u64)buf, (u64)done);
    mb_red_or_release(&mb->ready, 1ull << s);
    Job* j = b.job;
    const u64 t0 = gtime();
    unsigned ns = 32;
    while (!ld_acquire32(done)) {
        mb_release_taken();
        if (ld_relaxed_int(&j->status[0]) != 0) {
            *rc = fail_code(j);
            return 1;
        }
        if (gtime() - t0 > b.timeout_ns) {
            job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
            *rc = GPUMPI_ERR_TIMEOUT;
            return 1;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
    }
    *rc = MPI_SUCCESS;
    return 1;
}

// Leader: blocking send of an eager message without a request object.  Reads
// only the block's shared-memory copies of job state; the stamp and the slot
// claim are in flight together.  Returns 0 (before publishing anything) when
// the destination's mailbox is full.
__device__ int p2p_send_small(const void* buf, u64 bytes, int dest_job, int ctx, int me, int tag, int* rc) {
    BlockCtx& b = bctx();
    if (bytes <= INLINE_BYTES) {   // the payload travels in the header
        *rc = MPI_SUCCESS;
        return send_tiny(buf, (u32)bytes, dest_job, ctx, me, tag);
    }
    const bool bulk = leader_bulk_ok(buf, bytes);
    if (bytes > FAST_MSG_BYTES && !bulk) return 0;
    Mailbox* mb = mbox_of(dest_job);
    const u64 stamp = mb_atom_add(&mb->stamp, 1ull);   // a skipped stamp only leaves a gap
    // up to 64 aligned bytes are loaded now, while the atomics are in flight
    const bool pre = bytes <= 64 && ((uintptr_t)buf & 15) == 0;
    uint4 v[4];
    if (pre) {
#pragma unroll
        for (int k = 0; k < 4; k++)
            if ((u64)k * 16 < bytes) v[k] = ((const uint4*)buf)[k];
    }
    const int s = claim_slot_small(mb);
    if (s < 0) return 0;
    MsgHdr* h = &mb->hdr[s];
    *(int4*)h = make_int4(ctx, me, tag, 0);   // ctx, src, tag, kind = eager
    *(ulonglong2*)&h->bytes = make_ulonglong2(bytes, stamp);
    char* slot = b.eager + ((u64)dest_job * MB_SLOTS + s) * b.eager_bytes;
    *rc = MPI_SUCCESS;
    if (pre) {   // whole vectors: the slot holds at least 16 * ceil(bytes / 16) bytes
#pragma unroll
        for (int k = 0; k < 4; k++)
            if ((u64)k * 16 < bytes) ((uint4*)slot)[k] = v[k];
    } else if (bulk) {
        const u64 n16 = bytes & ~(u64)15;
        *rc = leader_bulk_copy(slot, (const char*)buf, n16);
        if (*rc) return 1;   // the job has failed; nothing is published
        for (u64 i = n16; i < bytes; i++) slot[i] = ((const char*)buf)[i];
    } else if (bytes) {
        leader_copy(slot, buf, bytes);
    }
    mb_red_or_release(&mb->ready, 1ull << s);
    return 1;
}

// ---------------------------------------------------------------- leader receives
// Receive matched message m into buf (capacity `bytes`) and take its slot
// (released at the leader's next idle moment, mb_take).  Returns 1 (done: *rc
// and *got set), or 0 when the request path must take it (nothing consumed).
__device__ int p2p_small_take(Mailbox* mb, const SmallMatch& m, void* buf, u64 bytes, int* rc, u64* got) {
    BlockCtx& b = bctx();
    const char* slots = b.eager + (u64)b.rank * MB_SLOTS * b.eager_bytes;
    const u64 n = m.bytes < bytes ? m.bytes : bytes;
    const bool bulk = leader_bulk_ok(buf, n);
    u32* rdv_done = nullptr;
    const char* rdv_src = nullptr;
    if (m.kind != 0) {
        // rendezvous: the leader pulls from the sender's buffer when the bulk engine applies
        const ulonglong2 h2 = mb_ld2(&mb->hdr[m.slot].rdv_src);
        rdv_src = (const char*)h2.x;
        rdv_done = (u32*)h2.y;
        if (!bulk || ((uintptr_t)rdv_src & 15) != 0) return 0;
    } else if (n > FAST_MSG_BYTES && !bulk) {
        return 0;
    }
    char* d = (char*)buf;
    *got = 0;
    if (m.kind == 0 && m.bytes <= INLINE_BYTES) {   // the payload is already in registers
        mb_take(mb, m.slot);
        tiny_store(d, m.pre, (u32)n);
        *rc = m.bytes > bytes ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
        *got = n;
        return 1;
    }
    if (bulk) {
        const u64 n16 = n & ~(u64)15;
        const char* src = rdv_src ? rdv_src : slots + (u64)m.slot * b.eager_bytes;
        *rc = leader_bulk_copy(d, src, n16);
        if (*rc) return 1;   // the job has failed; the slot stays claimed
        for (u64 i = n16; i < n; i++) d[i] = __ldcg(src + i);
    } else {
        const char* src = slots + (u64)m.slot * b.eager_bytes;
        u64 i = 0;
        if (((uintptr_t)d & 15) == 0) {
            copy_vec16<true>((uint4*)d, (const uint4*)src, n >> 4);
            i = n & ~(u64)15;
        } else if (((uintptr_t)d & 7) == 0) {
            for (; i + 8 <= n; i += 8) *(u64*)(d + i) = __ldcg((const u64*)(src + i));
        }
        for (; i < n; i++) d[i] = __ldcg(src + i);
    }
    if (rdv_done) {
        __threadfence();
        st_release32(rdv_done, 1u);
    }
    mb_take(mb, m.slot);
    *rc = m.bytes > bytes ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
    *got = n;
    return 1;
}

__device__ int p2p_small_take_st(int slot, int kind, u64 msg_bytes, int src, int tag, void* buf, u64 bytes,
                                 MPI_Status* st) {
    BlockCtx& b = bctx();
    Mailbox* mb = mbox_of(b.rank);
    SmallMatch m;
    m.slot = slot;
    m.src = src;
    m.tag = tag;
    m.kind = kind;
    m.bytes = msg_bytes;
    m.pre = make_ulonglong2(0ull, 0ull);   // not read: the message is not an inline one
    int rc = MPI_SUCCESS;
    u64 got = 0;
    if (!p2p_small_take(mb, m, buf, bytes, &rc, &got)) return LEADER_PASS;
    set_status(st, src, tag, rc, got);
    return rc;
}

// ---------------------------------------------------------------- lazy receives
// MPI_Irecv while no receive is posted on the block path and
// no send is deferred: the request waits in the block's FIFO of lazy receives
// (posting order) instead of being posted.  A progress pass takes one snapshot
// of the ready bits and lets every lazy receive, oldest first, take its oldest
// matching message from that snapshot, so matching follows posting order, as
// on the block path.  A message the leader cannot take (a rendezvous message
// into a local buffer, ...), and every block-path call that matches messages,
// first post all lazy receives on the block path, in order (lazy_materialize).

// Post every lazy receive on the block path, oldest first.
__device__ int lazy_materialize() {
    BlockCtx& b = bctx();
    const int n = b.lazy_n;
    if (n == 0) return MPI_SUCCESS;
    int idx[LAZY_MAX];
    for (int i = 0; i < n; i++) idx[i] = b.lazy[i];
    b.lazy_n = 0;
    RankPriv* p = b.priv;
    int first = MPI_SUCCESS;
    for (int i = 0; i < n; i++) {
        MPI_Request_impl* r = &p->reqs[idx[i]];
        r->state = RS_NEW;
        if (r->bytes && !is_global(r->buf)) {
            void* g = heap_alloc(&b.job->heap, r->bytes);
            if (!g) {
                r->state = RS_DONE;
                r->st_err = MPI_ERR_NO_MEM;
                if (!first) first = MPI_ERR_NO_MEM;
                continue;
            }
            r->buf = g;
            r->stage_alloc = 1;
        }
        Call call;
        call.op = OP_RECV_POST;
        call.a[0] = (u64)r;
        const int rc = block_call(call);
        if (rc && !first) first = rc;
    }
    return first;
}

// One progress pass over the lazy receives.  Returns 0 or an error code.
__device__ int lazy_progress() {
    BlockCtx& b = bctx();
    if (b.lazy_n == 0) return MPI_SUCCESS;
    Mailbox* mb = mbox_of(b.rank);
    u64 ready = mb_ld_acquire(&mb->ready);
    RankPriv* p = b.priv;
    int i = 0;
    while (i < b.lazy_n && ready) {
        MPI_Request_impl* r = &p->reqs[b.lazy[i]];
        SmallMatch m;
        if (!small_match(mb, ready, r->ctx, r->peer, r->tag, &m)) {
            i++;
            continue;
        }
        int rc = MPI_SUCCESS;
        u64 got = 0;
        if (!p2p_small_take(mb, m, r->buf, r->bytes, &rc, &got)) return lazy_materialize();
        ready &= ~(1ull << m.slot);
        r->st_source = m.src;
        r->st_tag = m.tag;
        r->st_bytes = got;
        r->st_err = rc;
        r->state = RS_DONE;
        for (int k = i + 1; k < b.lazy_n; k++) b.lazy[k - 1] = b.lazy[k];
        b.lazy_n--;
        if (rc && rc != MPI_ERR_TRUNCATE) return rc;
    }
    return MPI_SUCCESS;
}

// Leader: wait for lazy receive r.  On return r is done, or (after a
// materialisation) posted on the block path; 0 or an error code.
__device__ int lazy_wait(MPI_Request_impl* r) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    const u64 t0 = gtime();
    unsigned ns = 32;
    for (;;) {
        const int rc = lazy_progress();
        if (rc) return rc;
        if (r->state != RS_LAZY) return MPI_SUCCESS;
        // a deferred send needs the block path's progress: wait there
        if (!b.p2p_quiet) return lazy_materialize();
        mb_release_taken();
        if (ld_relaxed_int(&j->status[0]) != 0) return fail_code(j);
        if (gtime() - t0 > b.timeout_ns) {
            job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(ns);
        if (ns < 128) ns <<= 1;
    }
}

// Leader: blocking receive of a small eager message into r (r->buf may be
// local memory).  Returns 0 with *handled = 1 when done, 0 with *handled = 0
// when the block path must take over, or an error code.
__device__ int p2p_recv_fast(MPI_Request_impl* r, int* handled) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    RankPriv* p = b.priv;
    *handled = 0;
    // lazy receives were posted earlier and match first: the block path posts them, then r
    if (p->recv_head >= 0 || p->defer_head >= 0 || b.lazy_n) return MPI_SUCCESS;
    Mailbox* mb = mbox_of(b.rank);
    const u64 t0 = gtime();
    unsigned ns = 32;
    for (;;) {
        u64 ready = mb_ld_acquire(&mb->ready);
        int best = -1;
        u64 best_stamp = ~0ull;
        while (ready) {
            const int s = __ffsll((long long)ready) - 1;
            ready &= ready - 1;
            const MsgHdr* h = &mb->hdr[s];
            const int4 h0 = mb_ld4(h);   // ctx, src, tag, kind
            if (h0.x != r->ctx) continue;
            if (r->peer != MPI_ANY_SOURCE && h0.y != r->peer) continue;
            if (r->tag != MPI_ANY_TAG && h0.z != r->tag) continue;
            const u64 st = mb_ld(&h->stamp);
            if (st < best_stamp) {
                best_stamp = st;
                best = s;
            }
        }
        if (best >= 0) {
            const MsgHdr* h = &mb->hdr[best];
            const u64 bytes = mb_ld(&h->bytes);
            const int4 h0 = mb_ld4(h);
            if (h0.w != 0 || bytes > FAST_MSG_BYTES) return MPI_SUCCESS;   // block path
            const u64 n = bytes < r->bytes ? bytes : r->bytes;
            const char* src = eager_slot(j, b.rank, best);
            if (bytes <= INLINE_BYTES) {   // the payload is in the header
                const ulonglong2 w = mb_ld2(&h->inl);
                const char* pc = (const char*)&w;
                for (u64 i = 0; i < n; i++) ((char*)r->buf)[i] = pc[i];
            } else if (n) {   // the slot is 16-byte aligned; the destination may not be
                char* d = (char*)r->buf;
                u64 i = 0;
                if (((uintptr_t)d & 15) == 0)
                    for (; i + 16 <= n; i += 16) *(uint4*)(d + i) = __ldcg((const uint4*)(src + i));
                else if (((uintptr_t)d & 7) == 0)
                    for (; i + 8 <= n; i += 8) *(u64*)(d + i) = __ldcg((const u64*)(src + i));
                for (; i < n; i++) d[i] = __ldcg(src + i);
            }
            r->st_source = h0.y;
            r->st_tag = h0.z;
            r->st_bytes = n;
            r->st_err = bytes > r->bytes ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
            mb_take(mb, best);
            r->state = RS_DONE;
            *handled = 1;
            return MPI_SUCCESS;
        }
        mb_release_taken();
        if (job_aborted(j)) return fail_code(j);
        if (gtime() - t0 > j->timeout_ns) {
            job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(ns);
        if (ns < 128) ns <<= 1;
    }
}

}  // namespace gm
