// Internal data layout and primitives of the GB300 device MPI runtime.
//
// Execution model.  One MPI rank is one thread block of T threads (T a
// multiple of 32, >= 64).  The converted program's scalar code runs on thread
// 0 of the block (the leader).  The other T-1 threads wait on named barrier 1;
// every MPI call the leader makes is written to shared memory and executed by
// all T threads together (`block_call` / `dispatch`).  This replaces the
// one-thread-per-rank model of gpu_libs/gpu_main/main.cu:103-131, where every
// copy was a single-thread memcpy (gpu_libs/gpu_libc/cuda_mpi.cu:168).
//
// Memory.  All runtime state lives in plain device memory (HBM), never in
// managed memory, and synchronises with GPU-scope release/acquire operations.
// The reference kept it in managed memory with system-scope atomics
// (cuda_mpi.cuh:78-113, :459-533).
//
// Waiting.  Every spin-wait is bounded by the job's timeout (%globaltimer)
// and by the job's abort flag; on expiry the call returns an error code and
// the job is marked failed.  Nothing traps.
#pragma once

#include <stdint.h>
#include <stddef.h>
#include <cuda_runtime.h>

#include "mpi.cuh"

namespace gm {

typedef unsigned long long u64;
typedef unsigned int u32;

// ----------------------------------------------------------------- limits
constexpr int MB_SLOTS = 64;             // mailbox slots per receiving rank (one u64 mask)
constexpr int MAX_COMMS = 64;            // live communicator handles per rank
constexpr int MAX_GROUPS = 64;           // live group handles per rank
constexpr int MAX_DTYPES = 64;           // derived datatypes per rank
constexpr int STAGE_BYTES = 64 * 1024;   // per-rank scratch for staging local-memory buffers
constexpr int OUT_LINE_MAX = 1024;       // longest formatted line kept whole
constexpr int COLL_SCRATCH_BYTES = 64 * 1024;

// ----------------------------------------------------------------- calls
enum CallOp : int {
    OP_EXIT = 0,
    OP_SEND_START,
    OP_RECV_POST,
    OP_WAIT,
    OP_TEST,
    OP_PROBE,
    OP_BARRIER,
    OP_BCAST,
    OP_REDUCE,
    OP_ALLREDUCE,
    OP_GATHERV,
    OP_SCATTERV,
    OP_ALLGATHERV,
    OP_ALLTOALLV,
    OP_REDUCE_SCATTER_BLOCK,
    OP_SCAN,
    OP_COMM_SPLIT,
    OP_COMM_DUP,
    OP_MEMCPY,
    OP_MEMSET,
    OP_FINALIZE,
    OP_PARFOR,
    OP_NUM
};


// ----------------------------------------------------------------- p2p
// Header of a message waiting in a receiver's mailbox slot.
struct MsgHdr {
    int ctx;
    int src;            // sender's rank in the communicator
    int tag;
    int kind;           // 0 = eager (payload in the slot), 1 = rendezvous (payload at rdv_src)
    u64 bytes;
    u64 stamp;          // arrival order at this receiver
    const void* rdv_src;
    u32* rdv_done;      // sender's completion word for rendezvous
    u64 inl[2];         // the payload of an eager message of at most INLINE_BYTES
};
static_assert(sizeof(MsgHdr) == 64, "MsgHdr layout");
constexpr u64 INLINE_BYTES = 16;   // eager payloads up to this size travel in the header

// Per-receiver mailbox.  Senders claim a slot by setting its bit in `used`,
// fill the header (and the eager payload), then set the bit in `ready` with
// release semantics.  Only the receiver clears bits.  A job whose ranks all
// share one thread-block cluster keeps each rank's mailbox in its block's
// shared memory (distributed shared memory for the senders); every access
// therefore uses generic addresses (the mb_* primitives below).
struct alignas(128) Mailbox {
    u64 used;
    u64 pad0[15];
    u64 ready;
    u64 pad1[15];
    u64 stamp;
    u64 pad2[15];
    MsgHdr hdr[MB_SLOTS];
};

enum ReqKind : int { RK_FREE = 0, RK_SEND = 1, RK_RECV = 2 };
enum ReqState : int { RS_NEW = 0, RS_DEFERRED, RS_POSTED, RS_WAIT_RDV, RS_DONE, RS_LAZY };
constexpr int LAZY_MAX = 16;   // receives an MPI_Irecv may leave unposted (see lazy_progress)

}  // namespace gm

// Request object (MPI_Request is a pointer to it).  Pooled per rank.
struct MPI_Request_impl {
    int kind;
    int state;
    int peer;           // comm rank of destination / source (or MPI_ANY_SOURCE)
    int tag;
    int ctx;
    int peer_world;     // job rank of the destination (sends)
    int src_rank;       // own rank in the communicator (sends)
    int index;          // position in the rank's pool
    void* buf;          // engine-side buffer, always global memory
    void* user_buf;     // caller's buffer when it was staged (local memory), else == buf
    gm::u64 bytes;      // send size or receive capacity
    gm::u64 stage_alloc;// nonzero when buf came from the heap for staging
    volatile gm::u32 done;  // rendezvous completion, written by the receiver
    int next;           // link in the posted-receive / deferred-send list
    int st_source;
    int st_tag;
    int st_err;
    gm::u64 st_bytes;
    int persistent;
    int pad;
};

namespace gm {

// ----------------------------------------------------------------- collectives
// Buffers a rank exposes to its peers for one collective call.
struct Pub {
    const void* sbuf;
    void* rbuf;
    const int* scounts;
    const int* sdispls;
    const int* rcounts;
    const int* rdispls;
    long long a0;
    long long a1;
};

__device__ __forceinline__ Pub load_pub(const Pub* p) {
    Pub v;
    const unsigned long long* s = reinterpret_cast<const unsigned long long*>(p);
    unsigned long long* d = reinterpret_cast<unsigned long long*>(&v);
#pragma unroll
    for (int i = 0; i < 8; i++) d[i] = __ldcg(s + i);
    return v;
}

// Communicator state shared by all members.  `arrive`, `mid` and `depart`
// hold, per member, the sequence number of the latest collective the member
// reached the corresponding point of.  Each member writes only its own entry,
// so no collective needs an atomic read-modify-write.
struct alignas(128) CommShared {
    int size;
    int ctx;
    int* members;       // job rank of each member; nullptr means identity (WORLD)
    Pub* pub;           // [size]
    u64* arrive;        // [size]
    u64* mid;           // [size]
    u64* depart;        // [size]
    u64 split_ptr;      // scratch used while creating a child communicator
    int topo_ndims;     // Cartesian topology (0 = none)
    int topo_dims[8];
    int topo_periods[8];
    int self_member;    // a rank's MPI_COMM_SELF: members points here, at its job rank
};

}  // namespace gm

struct MPI_Comm_impl {
    int kind;           // 0 free, 1 live handle, 2 WORLD sentinel, 3 SELF sentinel
    int ctx;
    int size;
    int rank;
    int refcnt;
    int pad;
    gm::CommShared* cs;
    gm::u64 seq;        // collectives entered on this communicator
};

struct MPI_Group_impl {
    int kind;           // 0 free, 1 live, 2 WORLD sentinel, 3 EMPTY sentinel
    int n;
    int* ranks;         // job ranks, heap allocated (nullptr for identity)
    int refcnt;
    int pad;
};

struct MPI_Op_impl {
    int builtin;        // 0..11 for predefined operators, -1 for user functions
    int commute;
    MPI_User_function* fn;
};

namespace gm {

struct Heap;

// Per-rank state touched only by the rank's own block.
struct RankPriv {
    u32 rdv_done_small;            // completion word of the leader's blocking rendezvous send
    MPI_Request_impl* reqs;
    int nreqs;
    int free_head;
    int recv_head, recv_tail;      // posted, unmatched receives, in posting order
    int defer_head, defer_tail;    // sends waiting for a mailbox slot, in order
    int initialized, finalized;
    int errno_v;
    int opt_ind, opt_err, opt_opt, opt_pos;
    char* opt_arg;
    char* strtok_save;
    u64 rng;
    unsigned int rnd[34];          // rand() state: additive-feedback generator
    int rnd_i;
    int rnd_seeded;
    char* stage;                   // STAGE_BYTES of global scratch
    int stage_off;
    int exited;
    MPI_Comm_impl comms[MAX_COMMS];    // [0] = WORLD, [1] = SELF
    MPI_Group_impl groups[MAX_GROUPS];
    int dt_count[MAX_DTYPES];          // derived contiguous types: count of base
    int dt_base[MAX_DTYPES];
    int dt_used;
};

// Slab allocator instance (see gmalloc.cu).
struct Heap {
    char* base;
    u64 bytes;
    u32 npages;
    u32 pad;
    struct PageMeta* meta;        // [npages]
    u32* cls_pages;               // [NCLS * npages], 0xffffffff = empty entry
    u32* cls_count;               // [NCLS]
    u32* cls_hint;                // [NCLS * 32]
    u32* next_page;               // bump pointer (1 word)
    u32* large_head;              // free large runs, address order (page + 1, 0 = none)
    u32* large_lock;              // lock of that list
    u64* partial;                 // [NCLS] tagged stacks of pages with free chunks
    u32* stats;                   // [8] counters
};

// Host set-up of a heap's control words (one zeroed block of heap_ctl_bytes()).
__host__ size_t heap_ctl_bytes();
__host__ void heap_set_ctl(Heap& h, char* ctl);

// One MPI job (a converted program instance with its own MPI_COMM_WORLD).
struct HostCall;

struct Job {
    int id;
    int nranks;
    int first_slot;
    int threads;                  // threads per rank block
    int argc;
    int max_requests;
    char** argv;
    u64 timeout_ns;
    u64 eager_bytes;
    Mailbox* mbox;                // [nranks]
    char* eager;                  // [nranks * MB_SLOTS * eager_bytes]
    RankPriv* priv;               // [nranks]
    MPI_Request_impl* reqpool;    // [nranks * max_requests]
    char* stage;                  // [nranks * STAGE_BYTES]
    CommShared* world_cs;
    CommShared* self_cs;          // [nranks]
    char* arena;                  // bump arena for communicator state
    u64 arena_bytes;
    u64* arena_off;
    Heap heap;
    char* out;                    // formatted stdout text, appended in arrival order
    u64 out_bytes;
    u64* out_off;
    char* errout;                 // formatted stderr text
    u64* errout_off;
    char* coll_scratch;           // [nranks * COLL_SCRATCH_BYTES]
    int* status;                  // [0] abort flag, [1] first error code, [2] error rank, [3] ranks done,
                                  // [4] ranks finalized, [5] ctx counter, [6] exit code of any exit()
    int* retvals;                 // [nranks]
    char* err_msg;                // 256 bytes
    u64 t0_ns;                    // %globaltimer at launch
    HostCall* hcall;              // [nranks] mapped host memory, or null: no host service
    u64* cl_done;                 // [nranks] loop shares finished by a rank's helper blocks
};

// Device -> host calls (file I/O of converted programs).  One slot per rank in
// host memory mapped into the device: the rank's leader fills the request,
// publishes state = 1 with a system-scope release, and waits (bounded) for
// the launcher to answer with state = 2.  The launcher polls the slots while
// the kernel runs.
constexpr int HOSTCALL_DATA = 4096;
enum HostCallOp : u32 {
    HC_OPEN = 1,     // data: path '\0' mode '\0' -> ret: handle
    HC_CLOSE = 2,    // a0: handle
    HC_WRITE = 3,    // a0: handle, data[len] -> ret: bytes written
    HC_READ = 4,     // a0: handle, a1: bytes wanted (<= HOSTCALL_DATA) -> data[len], ret: bytes read
    HC_FLUSH = 5,    // a0: handle
    HC_SEEK = 6,     // a0: handle, a1: offset, a2: whence
    HC_TELL = 7,     // a0: handle -> ret: position
    HC_REMOVE = 8,   // data: path
};
struct alignas(64) HostCall {
    u32 state;       // 0 idle, 1 posted by the device, 2 answered by the host
    u32 op;
    long long a[3];
    long long ret;   // < 0: failed, err holds errno
    int err;
    u32 len;         // bytes in data (request or answer)
    char pad[16];
    char data[HOSTCALL_DATA];
};
static_assert(offsetof(HostCall, data) % 16 == 0, "HostCall data alignment");

// ---------------------------------------------------------------- serving runtime
// A server is one persistent cooperative launch: `nworkers` worker blocks,
// each a rank slot that runs one rank of an admitted job after another, and
// one admin block.  The host posts admission records into a ring in pinned
// host memory mapped into the device; the admin block (the only reader of
// that memory) hands each admitted job's ranks to their worker blocks through
// device memory, watches the running jobs and posts the ticket of each
// finished job into the completion ring.
constexpr int SERVE_RING = 256;       // records of each ring
constexpr int SERVE_MAX_JOBS = 256;   // jobs running at once
struct AdmitRec {
    Job* job;                         // the job's device record (in its memory, initialised)
    int slot_base;                    // rank r runs in rank slot slot_base + r
    int nranks;
    u64 ticket;
};
struct ServeRing {
    u64 sub_head;                     // admission records posted (host writes)
    u64 pad0[15];
    AdmitRec sub[SERVE_RING];
    u64 done_head;                    // completion records posted (device writes)
    u64 pad1[15];
    u64 done[SERVE_RING];             // tickets of finished jobs
    int stop;                         // host: end once every admitted job has finished
    int kill;                         // host: end now (idle workers leave)
};
struct ServeActive {
    Job* job;
    int nranks;
    int slot_base;
    u64 ticket;
};
struct ServerArgs {
    ServeRing* ring;                  // device address of the mapped ring
    u64* assign_seq;                  // [nworkers] assignment counter; ~0 = stop
    Job** assign_job;                 // [nworkers]
    int* assign_rank;                 // [nworkers]
    int* assign_slot;                 // [nworkers] rank slot of the assigned rank
    int* worker_sm;                   // [nworkers] SM each worker block runs on (written at start)
    const int* perm;                  // [nworkers] rank slot -> worker block (slots interleave the SMs)
    int* lost;                        // [nworkers] by rank slot: 1 = its block left (a rank called exit())
    ServeActive* active;              // [SERVE_MAX_JOBS] admin block's table
    int nworkers;
    int slot_base;                    // rank slot of worker block 0
};

// Where a thread block finds its job: slot -> (job, rank).
struct Launch {
    Job* jobs;
    int njobs;
    int nslots;
    int* slot_job;                // [nslots], -1 = idle
    int* slot_rank;               // [nslots]
    int slot_base;                // rank slot of block 0 (launches that run at once use disjoint ranges)
    int job_cluster;              // 1: the launch is one cluster, one block per rank, mailboxes in
                                  // shared memory (the job's rank r is the cluster's block r)
};


// ----------------------------------------------------------------- primitives
__device__ __forceinline__ u64 gtime() {
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Block barriers use the non-aligned `barrier.sync` form: the leader thread
// (lane 0 of warp 0) arrives from user code while lanes 1-31 of its warp
// arrive from the helper loop, which the aligned `bar.sync` does not allow.
__device__ __forceinline__ void bar_named(int id, int nthreads) {
    asm volatile("barrier.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
// Block-wide OR of a predicate (non-aligned barrier 3).
__device__ __forceinline__ int bar_or(int pred, int nthreads) {
    int r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, 3, %2, p;\n\tselp.s32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"(pred), "r"(nthreads)
        : "memory");
    return r;
}

__device__ __forceinline__ u64 ld_acquire(const u64* p) {
    u64 v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ u32 ld_acquire32(const u32* p) {
    u32 v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_acquire_int(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed_int(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(u64* p, u64 v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release32(u32* p, u32 v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ u64 atom_or_release(u64* p, u64 v) {
    u64 old;
    asm volatile("atom.release.gpu.global.or.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ u64 atom_or_acquire(u64* p, u64 v) {
    u64 old;
    asm volatile("atom.acquire.gpu.global.or.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
// Reductions that return nothing: the issuing thread does not wait for them.
__device__ __forceinline__ void red_or_release(u64* p, u64 v) {
    asm volatile("red.release.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_and_relaxed(u64* p, u64 v) {
    asm volatile("red.relaxed.gpu.global.and.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_and_release(u64* p, u64 v) {
    asm volatile("red.release.gpu.global.and.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ u64 ld_relaxed(const u64* p) {
    u64 v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ bool is_global(const void* p) { return __isGlobal(p) != 0; }


// Loads of data written by other rank blocks go through L2 (ld.global.cg), so
// a line this SM cached for an earlier message in the same slot or table entry
// can never be returned.
template <class T>
__device__ __forceinline__ T ldcg(const T* p) {
    if constexpr (sizeof(T) == 1) {
        unsigned char v = __ldcg(reinterpret_cast<const unsigned char*>(p));
        return *reinterpret_cast<T*>(&v);
    } else if constexpr (sizeof(T) == 2) {
        unsigned short v = __ldcg(reinterpret_cast<const unsigned short*>(p));
        return *reinterpret_cast<T*>(&v);
    } else if constexpr (sizeof(T) == 4) {
        unsigned int v = __ldcg(reinterpret_cast<const unsigned int*>(p));
        return *reinterpret_cast<T*>(&v);
    } else if constexpr (sizeof(T) == 8) {
        unsigned long long v = __ldcg(reinterpret_cast<const unsigned long long*>(p));
        return *reinterpret_cast<T*>(&v);
    } else if constexpr (sizeof(T) == 16 && alignof(T) >= 8) {
        ulonglong2 v;
        v.x = __ldcg(reinterpret_cast<const unsigned long long*>(p));
        v.y = __ldcg(reinterpret_cast<const unsigned long long*>(p) + 1);
        return *reinterpret_cast<T*>(&v);
    } else {
        T v;
        unsigned char* d = reinterpret_cast<unsigned char*>(&v);
        const unsigned char* s = reinterpret_cast<const unsigned char*>(p);
        for (unsigned i = 0; i < sizeof(T); i++) d[i] = __ldcg(s + i);
        return v;
    }
}

// Arguments of a collective call (all buffers global memory).
struct CollArgs {
    MPI_Comm_impl* comm;
    const void* sbuf;
    void* rbuf;
    const int* scounts;
    const int* sdispls;
    const int* rcounts;
    const int* rdispls;
    u64 count;          // elements (Bcast/Reduce/Allreduce/Scan) or per-block counts
    int ssize;          // element size of the send type
    int rsize;          // element size of the receive type
    MPI_Datatype dtype; // base type for reductions
    MPI_Op op;
    int opi;            // builtin operator index, -1 for a user function
    MPI_User_function* ufn;
    int root;
    int algo;           // 0 = choose automatically
    long long a0, a1;
};
// Arguments of one block-wide call, in shared memory.
struct Call {
    int op;
    int ret;
    union {
        u64 a[16];
        CollArgs ca;
    };
};

// Block-wide context, at offset 0 of dynamic shared memory.  `slot` comes
// first: converted programs index their per-rank globals with the int at the
// start of dynamic shared memory (include/gpumpi/global_vars.cuh).
struct BlockCtx {
    int slot;                     // rank slot, unique among all ranks running at once
    int rank;                     // rank in the job (MPI_COMM_WORLD rank)
    Job* job;
    RankPriv* priv;
    int T;                        // threads in the block
    int leader_mode;              // 1: thread 0 runs user code, others are helpers
    Call call;
    int bflag;                    // scratch broadcast words
    int bflag2;
    u64 bval;
    u64 bval2;
    int match_slot;
    int err;
    long long bcv;                // value broadcast by bcast()
    // Values thread 0 hands to the whole block (thread 0 alone reads and
    // writes rank-private state: requests, lists, communicator handles).
    struct Xfer {
        const void* src;
        void* dst;
        u64 bytes;
        int ctx, peer, tag, next;
        int slot, a, b, c;
    } x;
    // The communicator of the running collective, as read by thread 0.
    struct CommView {
        CommShared* shared;
        Pub* pub;
        u64* arrive;
        u64* mid;
        u64* depart;
        int P;
        int me;
        u64 seq;
    } cv;
    int in_call;                  // leader is inside block_call (helpers busy)
    int bulk_broken;              // a bulk pipeline failed with loads possibly in flight:
                                  // its barriers may not be initialised again
    // The leader's copies of what the blocking small-message paths read, so
    // that they touch no rank-private global state: a gpu-scope acquire drops
    // the SM's L1, after which every such read would be an L2 round trip.
    Mailbox* mbox;                // job's mailboxes (indexed by world rank)
    char* eager;                  // job's eager slots
    u64 eager_bytes;
    u64 timeout_ns;
    u64 slot_hint;                // `used` bits last seen at a destination
    u64 mb_taken;                 // slots of the own mailbox whose messages the leader took
                                  // and whose release waits for its next idle moment
    int world_ctx, world_size;
    int p2p_quiet;                // no posted receive and no deferred send
    unsigned api_calls;           // counts calls between checks of the abort word
    int lazy_n;                   // lazy receives (request indices), oldest first
    int lazy[LAZY_MAX];
    // the last communicator other than MPI_COMM_WORLD resolved by a leader-path
    // call (cleared when a communicator is freed): handle, context, the
    // caller's rank, size and member table
    const void* sc_handle;
    const int* sc_members;
    int sc_ctx, sc_me, sc_size;
    // A rank may be a cluster of cl_n thread blocks (cl_n = 1: one block).
    // Block cl_rank 0 runs the program; the others ("helper blocks") take
    // shares of its parallel loops.  The leader block writes a command into
    // a helper block's cl_cmd through distributed shared memory and arrives
    // on the helper's cl_go barrier; helpers report completion through the
    // job's cl_done counter of the rank in global memory, so that no helper
    // ever touches the leader block's shared memory.
    int mb_cluster;               // 1: mailboxes in the shared memory of the job's one cluster
    Mailbox* mb_local;            // this block's shared-memory mailbox (generic address)
    int cl_n;
    int cl_rank;
    int cl_released;              // leader: the helpers were told to exit
    u32 cl_phase;                 // leader: loops handed out; helper: commands taken
    u64 cl_go;                    // helper: mbarrier (count 1), arrived on by the leader block
    struct ClusterCmd {
        int op;                   // OP_PARFOR or OP_EXIT
        int pad;
        u64 a[3];                 // body, argument, iterations
    } cl_cmd;
};

static_assert(offsetof(BlockCtx, slot) == 0, "converted programs read the rank slot at offset 0");

// The mailbox of job rank r (global memory, or block r of the job's cluster).
__device__ __forceinline__ Mailbox* mbox_of(int r) {
    extern __shared__ __align__(16) char gm_dsmem[];
    const BlockCtx& b = *reinterpret_cast<const BlockCtx*>(gm_dsmem);
    if (!b.mb_cluster) return b.mbox + r;
    Mailbox* m;
    asm("mapa.u64 %0, %1, %2;" : "=l"(m) : "l"(b.mb_local), "r"(r));
    return m;
}
// Shared memory a block sets aside at the end of its dynamic shared memory for
// its mailbox when the job is one cluster.
constexpr int MB_SMEM_BYTES = (int)((sizeof(Mailbox) + 127) / 128 * 128);

// Dynamic shared memory of a rank block: BlockCtx, then (when the launch
// gave more) the bulk-copy area: mbarriers, then staging buffers.
constexpr int BCTX_BYTES = (int)((sizeof(BlockCtx) + 127) / 128 * 128);
constexpr int BULK_BAR_BYTES = 128;
constexpr int BULK_STAGES = 3;
constexpr u64 BULK_MIN_BYTES = 16 * 1024;   // blk_copy: smaller copies use vector loads
constexpr u64 BULK_SEG_MIN = 4 * 1024;      // multi-segment copies: average segment size for the bulk engine
__host__ __device__ constexpr size_t rank_smem_bytes(size_t stage) {
    return (size_t)BCTX_BYTES + (stage ? (size_t)BULK_BAR_BYTES + stage : 0);
}

__device__ __forceinline__ BlockCtx& bctx() {
    extern __shared__ __align__(16) char gm_dsmem[];
    return *reinterpret_cast<BlockCtx*>(gm_dsmem);
}

// Mailbox words and headers, by generic address: global memory, or the
// shared memory of a block of this cluster.  Loads are L2-coherent (relaxed,
// gpu scope) like ld.global.cg on global memory.
__device__ __forceinline__ u64 mb_ld(const u64* p) {
    u64 v;
    asm volatile("ld.relaxed.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int mb_ld_int(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Mailbox release/acquire: cluster scope when every rank of the job shares one
// cluster (its mailboxes and all its senders are in the cluster), else gpu.
__device__ __forceinline__ bool mb_in_cluster() { return bctx().mb_cluster != 0; }
__device__ __forceinline__ u64 mb_ld_acquire(const u64* p) {
    u64 v;
    if (mb_in_cluster()) asm volatile("ld.acquire.cluster.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    else asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int4 mb_ld4(const void* p) {
    int4 v;
    asm volatile("ld.relaxed.gpu.v4.s32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p)
                 : "memory");
    return v;
}
__device__ __forceinline__ ulonglong2 mb_ld2(const void* p) {
    ulonglong2 v;
    asm volatile("ld.relaxed.gpu.v2.u64 {%0,%1}, [%2];" : "=l"(v.x), "=l"(v.y) : "l"(p) : "memory");
    return v;
}
// The slot masks change one bit at a time, with 32-bit atomics on the half of
// the 64-bit word that holds the bit: on distributed shared memory the 64-bit
// bitwise atomics lost updates when several blocks hit one word (a bounded
// probe on GB300 received 2.5-3.0 thousand of 14 thousand messages through the
// 64-bit forms and all of them through the 32-bit forms).
__device__ __forceinline__ u32* mb_half(u64* p, u64 bit) {
    return reinterpret_cast<u32*>(p) + ((bit >> 32) ? 1 : 0);
}
__device__ __forceinline__ u32 mb_bit32(u64 bit) { return (bit >> 32) ? (u32)(bit >> 32) : (u32)bit; }
// Set one bit; returns the old value of the bit's half in its place (the other half reads 0).
__device__ __forceinline__ u64 mb_atom_or_acquire(u64* p, u64 bit) {
    u32 old;
    if (mb_in_cluster())
        asm volatile("atom.acquire.cluster.or.b32 %0, [%1], %2;" : "=r"(old) : "l"(mb_half(p, bit)),
                     "r"(mb_bit32(bit)) : "memory");
    else
        asm volatile("atom.acquire.gpu.or.b32 %0, [%1], %2;" : "=r"(old) : "l"(mb_half(p, bit)), "r"(mb_bit32(bit))
                     : "memory");
    return (bit >> 32) ? ((u64)old << 32) : (u64)old;
}
// Arrival counter (32 bits: stamps of one receiver's messages within a job).
__device__ __forceinline__ u64 mb_atom_add(u64* p, u64 v) {
    u32 old;
    asm volatile("atom.relaxed.gpu.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(reinterpret_cast<u32*>(p)), "r"((u32)v)
                 : "memory");
    return (u64)old;
}
__device__ __forceinline__ void mb_red_or_release(u64* p, u64 bit) {
    if (mb_in_cluster())
        asm volatile("red.release.cluster.or.b32 [%0], %1;" ::"l"(mb_half(p, bit)), "r"(mb_bit32(bit)) : "memory");
    else
        asm volatile("red.release.gpu.or.b32 [%0], %1;" ::"l"(mb_half(p, bit)), "r"(mb_bit32(bit)) : "memory");
}
// Clear one bit: mask = ~bit.
__device__ __forceinline__ void mb_red_and_relaxed(u64* p, u64 mask) {
    const u64 bit = ~mask;
    asm volatile("red.relaxed.gpu.and.b32 [%0], %1;" ::"l"(mb_half(p, bit)), "r"(~mb_bit32(bit)) : "memory");
}
__device__ __forceinline__ void mb_red_and_release(u64* p, u64 mask) {
    const u64 bit = ~mask;
    if (mb_in_cluster())
        asm volatile("red.release.cluster.and.b32 [%0], %1;" ::"l"(mb_half(p, bit)), "r"(~mb_bit32(bit)) : "memory");
    else
        asm volatile("red.release.gpu.and.b32 [%0], %1;" ::"l"(mb_half(p, bit)), "r"(~mb_bit32(bit)) : "memory");
}

// Clear several bits of a slot mask, release (one 32-bit atomic per half that has bits).
__device__ __forceinline__ void mb_release_bits(u64* p, u64 bits) {
    u32* w = reinterpret_cast<u32*>(p);
    const u32 lo = (u32)bits, hi = (u32)(bits >> 32);
    if (mb_in_cluster()) {
        if (lo) asm volatile("red.release.cluster.and.b32 [%0], %1;" ::"l"(w), "r"(~lo) : "memory");
        if (hi) asm volatile("red.release.cluster.and.b32 [%0], %1;" ::"l"(w + 1), "r"(~hi) : "memory");
    } else {
        if (lo) asm volatile("red.release.gpu.and.b32 [%0], %1;" ::"l"(w), "r"(~lo) : "memory");
        if (hi) asm volatile("red.release.gpu.and.b32 [%0], %1;" ::"l"(w + 1), "r"(~hi) : "memory");
    }
}

// Slots of the leader's own mailbox.  A message the leader takes has its
// ready bit cleared at once (relaxed: the slot stays claimed), while the
// release of the slot itself -- a release operation, whose fence would wait
// for every earlier memory operation of the thread -- is put off until the
// leader next waits (mb_release_taken: on a poll that finds nothing, before a
// block-path call, or once MB_TAKEN_MAX slots are held), off the path between
// a message's arrival and the caller's next operation.
constexpr int MB_TAKEN_MAX = 16;
__device__ __forceinline__ void mb_release_taken() {
    BlockCtx& b = bctx();
    if (b.mb_taken) {
        mb_release_bits(&mbox_of(b.rank)->used, b.mb_taken);
        b.mb_taken = 0;
    }
}
__device__ __forceinline__ void mb_take(Mailbox* mb, int s) {
    BlockCtx& b = bctx();
    mb_red_and_relaxed(&mb->ready, ~(1ull << s));
    b.mb_taken |= 1ull << s;
    if (__popcll(b.mb_taken) >= MB_TAKEN_MAX) mb_release_taken();
}

// Intra-call barrier of all threads of the rank block.
__device__ __forceinline__ void bsync() { bar_named(2, bctx().T); }

// Broadcast a value computed on thread 0 to every thread of the block.  The
// leading barrier guarantees all threads have consumed the previous value.
__device__ __forceinline__ long long bcast(long long x, int tid) {
    BlockCtx& b = bctx();
    bsync();
    if (tid == 0) b.bcv = x;
    bsync();
    return b.bcv;
}
__device__ __forceinline__ long long pack2(int hi, int lo) {
    return (long long)(((unsigned long long)(unsigned)hi << 32) | (unsigned)lo);
}
__device__ __forceinline__ int unpack_hi(long long v) { return (int)((unsigned long long)v >> 32); }
__device__ __forceinline__ int unpack_lo(long long v) { return (int)(unsigned)(unsigned long long)v; }

// ----------------------------------------------------------------- job status
__device__ __forceinline__ bool job_aborted(const Job* j) {
    return ld_acquire_int(&j->status[0]) != 0;
}
// Record the first error of the job (code, rank, message) and raise the abort flag.
__device__ void job_fail(Job* j, int rank, int code, const char* msg);
__device__ int fail_code(Job* j);

// Bounded wait helpers.  Return MPI_SUCCESS, GPUMPI_ERR_TIMEOUT or GPUMPI_ERR_ABORTED.
__device__ int wait_ge(const u64* addr, u64 target);
__device__ int wait_flags_ge(const u64* flags, int n, u64 target, int skip, int tid, int T);
__device__ int wait_u32_nonzero(const volatile u32* addr);

// ----------------------------------------------------------------- copies
// Block-cooperative copy of n bytes between global buffers.
__device__ void blk_copy(void* dst, const void* src, u64 n, int tid, int T);

// ---- bulk asynchronous copies (cp.async.bulk global -> shared -> global) ----
// One thread drives a ring of BULK_STAGES staging buffers: a chunk is loaded
// with cp.async.bulk into a stage (completion counted on the stage's
// mbarrier), then stored from the stage with a bulk store; up to
// BULK_STAGES - 1 loads are in flight while stores drain asynchronously.  Addresses and sizes
// must be multiples of 16 bytes.  Every wait is bounded by the job timeout.
__device__ u32 bulk_stage_bytes();     // staging bytes of this block (0: none)
struct BulkPipe {
    char* stage;
    u64* bars;
    u32 chunk;                 // bytes per stage
    u64 issued, stored;        // chunk counters
    char* dst_of[BULK_STAGES];
    u32 len_of[BULK_STAGES];
    int err;
    __device__ bool begin();                  // false: no staging area
    __device__ bool push(char* dst, const char* src, u64 n);   // queue a 16-byte aligned span
    __device__ int finish();                  // all stores complete; 0 or an error code
    __device__ bool retire();
};
__device__ void blk_memset(void* dst, int c, u64 n, int tid, int T);
// Same, using only the 32 lanes of one warp.
__device__ void warp_copy(void* dst, const void* src, u64 n, int lane);

// ----------------------------------------------------------------- leader side
__device__ int block_call(Call& c);
__device__ void helper_loop();
__device__ int dispatch_all(int tid);   // executed by every thread of the block

// Staging of local-memory buffers (leader thread only).
__device__ void* stage_temp(int bytes);
__device__ void stage_reset();

// Resolve a handle to the calling rank's communicator object.
__device__ MPI_Comm_impl* comm_resolve(MPI_Comm c);
__device__ __forceinline__ int comm_world_rank(const MPI_Comm_impl* c, int r) {
    return c->cs->members ? __ldcg(&c->cs->members[r]) : r;
}

// datatypes / operators
// The size of every basic datatype, packed at compile time from the datatype
// list (enum order) as 3-bit base-2 logarithms, so that a size is a shift of
// a constant rather than a call or a table load.
#define GPUMPI_SIZE_F(name, type) (unsigned)sizeof(type)
#define GPUMPI_SIZE_SEP ,
constexpr unsigned kBasicSizes[] = {GPUMPI_TYPES_LIST(GPUMPI_SIZE_F, GPUMPI_SIZE_SEP)};
#undef GPUMPI_SIZE_F
#undef GPUMPI_SIZE_SEP
constexpr int kNumBasic = (int)(sizeof(kBasicSizes) / sizeof(kBasicSizes[0]));
static_assert(kNumBasic == GPUMPI_NUM_BASIC_TYPES, "datatype list and enum differ");
static_assert(kNumBasic <= 42, "two words of packed sizes");
constexpr int size_lg2(unsigned v) { return v <= 1 ? 0 : 1 + size_lg2(v >> 1); }
constexpr bool sizes_ok() {
    for (int i = 0; i < kNumBasic; i++)
        if (kBasicSizes[i] == 0 || (kBasicSizes[i] & (kBasicSizes[i] - 1)) != 0 || kBasicSizes[i] > 64) return false;
    return true;
}
static_assert(sizes_ok(), "basic datatype sizes are powers of two up to 64 bytes");
constexpr u64 pack_size_lg2(int from) {
    u64 w = 0;
    for (int i = 0; i < 21 && from + i < kNumBasic; i++) w |= (u64)size_lg2(kBasicSizes[from + i]) << (3 * i);
    return w;
}
constexpr u64 kSizeLg2Lo = pack_size_lg2(0), kSizeLg2Hi = pack_size_lg2(21);

// Size in bytes of basic datatype t, 0 <= t < GPUMPI_NUM_BASIC_TYPES.
__device__ __forceinline__ int basic_size(int t) {
    const bool lo = t < 21;
    const u64 w = lo ? kSizeLg2Lo : kSizeLg2Hi;
    return 1 << (int)((w >> (3 * (lo ? t : t - 21))) & 7);
}

__device__ int dtype_size(MPI_Datatype t);
__device__ int dtype_base(MPI_Datatype t, int* mult);
__device__ int op_check(MPI_Op op, MPI_Datatype t);
struct Pub;
// Rank-order fold of elements [lo, hi): out[i - lo] = acc with acc = in_0[i];
// acc = op(in_q[i], acc) for q = 1..nin-1, where in_q = pub[q].sbuf + in_off bytes.
__device__ bool fold_range_push(int opi, MPI_Datatype base, const Pub* pub, int nin, u64 lo, u64 hi, int tid,
                                int T);
__device__ void fold_range(int opi, MPI_User_function* ufn, MPI_Datatype base, int esize, void* out, const Pub* pub, int nin,
                           u64 in_off, u64 lo, u64 hi, int tid, int T);

// p2p engine (block-cooperative)
__device__ int p2p_send_start(MPI_Request_impl* r, int tid, int T);
constexpr u64 FAST_MSG_BYTES = 1024;   // eager messages the leader moves alone
constexpr u64 SMALL_BULK_MIN = 512;    // leader copies from this size go through the bulk engine
// Blocking send/receive of an eager message by the leader, without a request
// object: up to FAST_MSG_BYTES always, up to the eager size when the user
// buffer is global, 16-byte aligned and the block has a bulk staging area.
// ctx is the communicator's context, me the caller's rank in it (the source
// the receiver matches), dest_job the destination's job rank and source a
// rank of the communicator (or MPI_ANY_SOURCE).  Return 1 when done (*rc
// set), 0 when the request path must take the call.
__device__ int p2p_send_small(const void* buf, u64 bytes, int dest_job, int ctx, int me, int tag, int* rc);
__device__ int p2p_send_rdv_small(const void* buf, u64 bytes, int dest_job, int ctx, int me, int tag, int* rc);
__device__ int lazy_materialize();
__device__ int lazy_progress();
__device__ int lazy_wait(MPI_Request_impl* r);
__device__ bool p2p_send_rdv_fast(MPI_Request_impl* r);
__device__ int rdv_wait_leader(MPI_Request_impl* r);
__device__ bool p2p_send_fast(MPI_Request_impl* r);
__device__ int p2p_recv_fast(MPI_Request_impl* r, int* handled);
__device__ int p2p_recv_post(MPI_Request_impl* r, int tid, int T);
__device__ int p2p_progress(int tid, int T, int* did_work);
__device__ int p2p_wait(MPI_Request_impl* r, int tid, int T, int blocking);
__device__ int p2p_probe(int source, int tag, int ctx, int blocking, MPI_Status* st, int tid, int T);

// collective engine (block-cooperative); all buffers are global memory


__device__ int coll_barrier(MPI_Comm_impl* c, int tid, int T);
__device__ int coll_bcast(const CollArgs& a, int tid, int T);
__device__ int coll_reduce(const CollArgs& a, int tid, int T);
__device__ int coll_allreduce(const CollArgs& a, int tid, int T);
__device__ int coll_gatherv(const CollArgs& a, int tid, int T);
__device__ int coll_scatterv(const CollArgs& a, int tid, int T);
__device__ int coll_allgatherv(const CollArgs& a, int tid, int T);
__device__ int coll_alltoallv(const CollArgs& a, int tid, int T);
__device__ int coll_alltoall(const CollArgs& a, int tid, int T);
__device__ int coll_reduce_scatter_block(const CollArgs& a, int tid, int T);
__device__ int coll_scan(const CollArgs& a, int exclusive, int tid, int T);
// Launch-ordered forms for host plans whose calls touch disjoint memory (no
// arrive/depart flags; `pub` is the call's buffer table, one entry per rank).
__device__ int coll_lo_bcast(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T);
__device__ int coll_lo_reduce(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T);
__device__ int coll_lo_allreduce(const CollArgs& a, const Pub* pub, int P, int me, int tid, int T);
__device__ int coll_lo_alltoall(const CollArgs& a, const Pub* pub, int P, int me, int gather, int tid, int T);
__device__ int comm_split_block(MPI_Comm_impl* parent, int color, int key, MPI_Comm_impl** out,
                                int tid, int T);

// heap
__device__ void* heap_alloc(Heap* h, u64 bytes);
__device__ void heap_free(Heap* h, void* p);
__device__ u64 heap_usable_size(Heap* h, void* p);

// cluster ranks (csrc/cluster.cu)
__device__ void cluster_setup(int tid);                       // every block of a cluster, at start
__device__ int cluster_parfor(void (*body)(long, void*), void* arg, long n, int tid, int T);
__device__ void cluster_release();                            // leader block: helpers may exit
__device__ void cluster_helper_loop();                        // helper blocks

// serving runtime (csrc/server.cu)
__device__ void server_admin(const ServerArgs& A);
__device__ bool server_take(const ServerArgs& A, int w, u64* seen, Job** job, int* rank, int* slot);
__device__ void rank_block_setup(Job* job, int rank, int slot);   // every thread; one-block rank

// rank lifecycle
__device__ void rank_init(int tid, int T);
__device__ void rank_finish(int rc);
__device__ int out_write(Job* j, int stream, const char* s, int n);   // stream 1 stdout, 2 stderr
__device__ void rank_exit_now(int status);   // end the calling rank (leader thread) immediately

}  // namespace gm
