// Leader-only small-message pieces shared by the API layer (api_p2p.cu) and
// the point-to-point engine (p2p.cu).  They are inlined into the blocking
// MPI_Send / MPI_Recv / MPI_Sendrecv entry points: a message of a few bytes
// then costs the leader thread one call from the program and no further
// calls, since a call across translation units saves and restores registers
// through local memory and, for a single thread, the instructions of the path
// are its latency.
#pragma once
#include "rt.cuh"

namespace gm {

// Result of a leader-path function that leaves the call to the request path
// (no MPI return code has this value).
constexpr int LEADER_PASS = (int)0x80000000;

// ---------------------------------------------------------------- slot claim
// Leader: claim a free slot of mailbox mb (first guess from the bits last seen
// there), or -1 when it is full.  The claim is an acquire: the slot is written
// only after its previous receiver released it.
static __device__ __forceinline__ int claim_slot_small(Mailbox* mb) {
    BlockCtx& b = bctx();
    u64 used = b.slot_hint;
    for (int tries = 0;; tries++) {
        if (~used == 0) {
            if (tries) return -1;
            used = mb_ld(&mb->used);
            if (~used == 0) return -1;
        }
        const int s = __ffsll((long long)~used) - 1;
        const u64 bit = 1ull << s;
        const u64 old = mb_atom_or_acquire(&mb->used, bit);   // the bit's 32-bit half
        if (!(old & bit)) {
            b.slot_hint = (used & ((bit >> 32) ? 0xffffffffull : ~0xffffffffull)) | old | bit;
            return s;
        }
        used |= old | bit;
    }
}

// ---------------------------------------------------------------- payloads in the header
// Up to INLINE_BYTES of payload as two little-endian words.  Aligned 4, 8 and
// 16-byte payloads are one access; other sizes are assembled byte by byte in
// registers.  No call: a call on this path would make the caller keep its
// live values in callee-saved registers, saved and restored through local
// memory on every MPI_Send and MPI_Recv.
__device__ __forceinline__ ulonglong2 tiny_load(const void* buf, u32 n) {
    const uintptr_t a = (uintptr_t)buf;
    if (n == 8 && (a & 7) == 0) return make_ulonglong2(*(const u64*)buf, 0ull);
    if (n == 4 && (a & 3) == 0) return make_ulonglong2((u64)*(const u32*)buf, 0ull);
    if (n == 16 && (a & 15) == 0) return *(const ulonglong2*)buf;
    u64 lo = 0, hi = 0;
    const unsigned char* p = (const unsigned char*)buf;
    for (u32 i = 0; i < n && i < INLINE_BYTES; i++) {
        const u64 v = p[i];
        if (i < 8) lo |= v << (8 * i);
        else hi |= v << (8 * (i - 8));
    }
    return make_ulonglong2(lo, hi);
}
__device__ __forceinline__ void tiny_store(void* buf, ulonglong2 w, u32 n) {
    const uintptr_t a = (uintptr_t)buf;
    if (n == 8 && (a & 7) == 0) {
        *(u64*)buf = w.x;
    } else if (n == 4 && (a & 3) == 0) {
        *(u32*)buf = (u32)w.x;
    } else if (n == 16 && (a & 15) == 0) {
        *(ulonglong2*)buf = w;
    } else {
        unsigned char* p = (unsigned char*)buf;
        for (u32 i = 0; i < n && i < INLINE_BYTES; i++)
            p[i] = (unsigned char)(i < 8 ? w.x >> (8 * i) : w.y >> (8 * (i - 8)));
    }
}

// Leader: blocking send of an eager message of at most INLINE_BYTES, the
// payload in the header.  The arrival stamp, the payload load and the slot
// claim are in flight together; false (nothing published) when the
// destination's mailbox is full.
static __device__ __forceinline__ bool send_tiny(const void* buf, u32 bytes, int dest_job, int ctx, int me, int tag) {
    Mailbox* mb = mbox_of(dest_job);
    const u64 stamp = mb_atom_add(&mb->stamp, 1ull);   // a skipped stamp only leaves a gap
    const ulonglong2 w = tiny_load(buf, bytes);
    const int s = claim_slot_small(mb);
    if (s < 0) return false;
    MsgHdr* h = &mb->hdr[s];
    *(int4*)h = make_int4(ctx, me, tag, 0);   // ctx, src, tag, kind = eager
    *(ulonglong2*)&h->bytes = make_ulonglong2(bytes, stamp);
    *(ulonglong2*)&h->inl = w;
    mb_red_or_release(&mb->ready, 1ull << s);
    return true;
}

// ---------------------------------------------------------------- matching
// A message of this rank's mailbox that matched (ctx, source, tag).
struct SmallMatch {
    int slot, src, tag, kind;
    u64 bytes;
    ulonglong2 pre;   // the payload of an eager message of at most INLINE_BYTES
};

// The oldest message among the `ready` slots matching (ctx, source, tag).  The
// header's first 32 bytes are read as two vectors, the first 16 payload bytes
// with them.
static __device__ __forceinline__ bool small_match(Mailbox* mb, u64 ready, int ctx, int source, int tag,
                                                   SmallMatch* m) {
    u64 best_stamp = ~0ull;
    m->slot = -1;
    while (ready) {
        const int s = __ffsll((long long)ready) - 1;
        ready &= ready - 1;
        const int4 h0 = mb_ld4(&mb->hdr[s]);
        const ulonglong2 h1 = mb_ld2(&mb->hdr[s].bytes);
        const ulonglong2 p0 = mb_ld2(&mb->hdr[s].inl);   // the payload when bytes <= INLINE_BYTES
        if (h0.x != ctx) continue;
        if (source != MPI_ANY_SOURCE && h0.y != source) continue;
        if (tag != MPI_ANY_TAG && h0.z != tag) continue;
        if (h1.y < best_stamp) {
            best_stamp = h1.y;
            m->slot = s;
            m->src = h0.y;
            m->tag = h0.z;
            m->kind = h0.w;
            m->bytes = h1.x;
            m->pre = p0;
        }
    }
    return m->slot >= 0;
}

// Receive matched message m of this rank's mailbox into buf (capacity
// `bytes`): 1 when done (*rc and *got set), 0 when the request path must take
// it (nothing consumed).  (p2p.cu)
__device__ int p2p_small_take(Mailbox* mb, const SmallMatch& m, void* buf, u64 bytes, int* rc, u64* got);
// The same for the message in `slot` of this rank's mailbox, with the status
// filled in: the MPI result, or LEADER_PASS when the request path must take it.  The
// match is passed by value so that the inline path keeps it in registers.
__device__ int p2p_small_take_st(int slot, int kind, u64 msg_bytes, int src, int tag, void* buf, u64 bytes,
                                 MPI_Status* st);

__device__ __forceinline__ void set_status(MPI_Status* st, int src, int tag, int err, u64 got) {
    if (st) {
        st->MPI_SOURCE = src;
        st->MPI_TAG = tag;
        st->MPI_ERROR = err;
        st->gpumpi_count_lo = (int)(got & 0xffffffffu);
        st->gpumpi_count_hi = (int)(got >> 32);
    }
}

// Leader: blocking receive without a request object.  A message of at most
// INLINE_BYTES is taken here from the registers its header was read into;
// anything larger goes to p2p_small_take_st.  Returns the MPI result (of the
// receive, or of a failed job), or LEADER_PASS when the request path must take
// the message.
static __device__ __forceinline__ int recv_small(void* buf, u64 bytes, int ctx, int source, int tag, MPI_Status* st) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    Mailbox* mb = mbox_of(b.rank);
    const u64 t0 = gtime();
    unsigned ns = 32;
    for (unsigned it = 0;; it++) {
        // acquire on every poll: nothing read after it comes from L1 anyway
        const u64 ready = mb_ld_acquire(&mb->ready);
        SmallMatch m;
        if (ready && small_match(mb, ready, ctx, source, tag, &m)) {
            if (m.kind != 0 || m.bytes > INLINE_BYTES)
                return p2p_small_take_st(m.slot, m.kind, m.bytes, m.src, m.tag, buf, bytes, st);
            const u64 got = m.bytes < bytes ? m.bytes : bytes;
            mb_take(mb, m.slot);
            tiny_store(buf, m.pre, (u32)got);
            const int rc = m.bytes > bytes ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
            set_status(st, m.src, m.tag, rc, got);
            return rc;
        }
        mb_release_taken();
        // the abort word and the clock every 8th poll: a poll of a mailbox in
        // shared memory is much shorter than a load of the abort word
        if ((it & 7u) == 7u) {
            if (ld_relaxed_int(&j->status[0]) != 0) return fail_code(j);
            if (gtime() - t0 > b.timeout_ns) {
                job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
                return GPUMPI_ERR_TIMEOUT;
            }
        }
        // the first polls follow each other at once (a reply usually comes
        // within a few microseconds), later ones back off
        if (it >= 16) {
            __nanosleep(ns);
            if (ns < 128) ns <<= 1;
        }
    }
}

}  // namespace gm
