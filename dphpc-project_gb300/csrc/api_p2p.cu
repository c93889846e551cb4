// Leader-side entry points of the point-to-point API, environment and
// datatype calls.  These run on the rank's leader thread; block-wide work is
// handed to the whole rank block through block_call().
//
// Buffers in the leader's local memory (stack arrays and scalars of the
// converted program, e.g. `MPI_Bcast(&n, ...)` in toolchain_tests/pi/cpi.c) are
// not addressable by the helper threads, so they are staged through global
// memory; the reference instead copied non-global buffers into malloc'd bounce
// buffers (gpu_libs/gpu_libc/cuda_mpi.cu:183-194).
#include "rt.cuh"
#include "p2p_small.cuh"

using namespace gm;

extern __device__ MPI_Comm_impl gm_world_sentinel;

namespace gm {

__device__ int aborted_code() { return fail_code(bctx().job); }

__device__ MPI_Request_impl* req_alloc() {
    RankPriv* p = bctx().priv;
    int i = p->free_head;
    if (i < 0) return nullptr;
    MPI_Request_impl* r = &p->reqs[i];
    p->free_head = r->next;
    r->next = -1;
    r->kind = RK_FREE;
    r->state = RS_NEW;
    r->stage_alloc = 0;
    r->done = 0;
    r->st_source = MPI_ANY_SOURCE;
    r->st_tag = MPI_ANY_TAG;
    r->st_err = MPI_SUCCESS;
    r->st_bytes = 0;
    r->persistent = 0;
    return r;
}

__device__ void req_release(MPI_Request_impl* r) {
    RankPriv* p = bctx().priv;
    r->kind = RK_FREE;
    r->state = RS_NEW;
    r->next = p->free_head;
    p->free_head = r->index;
}

__device__ bool req_valid(MPI_Request_impl* r) {
    RankPriv* p = bctx().priv;
    return r >= p->reqs && r < p->reqs + p->nreqs && r->kind != RK_FREE;
}

}  // namespace gm

static __device__ void fill_status(MPI_Status* st, const MPI_Request_impl* r) {
    if (!st) return;
    st->MPI_SOURCE = r->st_source;
    st->MPI_TAG = r->st_tag;
    st->MPI_ERROR = r->st_err;
    st->gpumpi_count_lo = (int)(r->st_bytes & 0xffffffffu);
    st->gpumpi_count_hi = (int)(r->st_bytes >> 32);
}

static __device__ void empty_status(MPI_Status* st) {
    if (!st) return;
    st->MPI_SOURCE = MPI_ANY_SOURCE;
    st->MPI_TAG = MPI_ANY_TAG;
    st->MPI_ERROR = MPI_SUCCESS;
    st->gpumpi_count_lo = 0;
    st->gpumpi_count_hi = 0;
}

// The abort word is read (relaxed) on every 16th call: an acquire load here
// would drop the leader's cached rank state from L1 on every call.  Waits read
// it on every poll, so a rank blocked anywhere still sees an abort at once.
__device__ __forceinline__ bool api_abort_check(BlockCtx& b) {
    if ((++b.api_calls & 15u) != 0) return false;
    return ld_relaxed_int(&b.job->status[0]) != 0;
}

#define API_ENTER()                                         \
    BlockCtx& b = bctx();                                   \
    if (api_abort_check(b)) return aborted_code();

// ---------------------------------------------------------------- environment
__device__ int MPI_Init(int* argc, char*** argv) {
    (void)argc;
    (void)argv;
    bctx().priv->initialized = 1;
    return MPI_SUCCESS;
}

__device__ int MPI_Init_thread(int* argc, char*** argv, int required, int* provided) {
    (void)required;
    if (provided) *provided = MPI_THREAD_SINGLE;
    return MPI_Init(argc, argv);
}

__device__ int MPI_Initialized(int* flag) {
    *flag = bctx().priv->initialized;
    return MPI_SUCCESS;
}

__device__ int MPI_Finalize(void) {
    API_ENTER();
    Call c;
    c.op = OP_FINALIZE;
    int rc = block_call(c);
    b.priv->finalized = 1;
    atomicAdd(&b.job->status[4], 1);
    return rc;
}

__device__ int MPI_Finalized(int* flag) {
    *flag = bctx().priv->finalized;
    return MPI_SUCCESS;
}

__device__ int MPI_Abort(MPI_Comm comm, int errorcode) {
    (void)comm;
    BlockCtx& b = bctx();
    job_fail(b.job, b.rank, GPUMPI_ERR_ABORTED, "MPI_Abort called");
    rank_exit_now(errorcode ? errorcode : 1);
    return MPI_SUCCESS;
}

__device__ int MPI_Get_processor_name(char* name, int* resultlen) {
    const char host[] = "gb300-rank-block";
    int i = 0;
    for (; host[i]; i++) name[i] = host[i];
    name[i] = 0;
    *resultlen = i;
    return MPI_SUCCESS;
}

__device__ int MPI_Error_string(int errorcode, char* string, int* resultlen) {
    const char* s = "MPI error";
    switch (errorcode) {
        case MPI_SUCCESS: s = "success"; break;
        case MPI_ERR_BUFFER: s = "invalid buffer"; break;
        case MPI_ERR_COUNT: s = "invalid count"; break;
        case MPI_ERR_TYPE: s = "invalid datatype"; break;
        case MPI_ERR_TAG: s = "invalid tag"; break;
        case MPI_ERR_COMM: s = "invalid communicator"; break;
        case MPI_ERR_RANK: s = "invalid rank"; break;
        case MPI_ERR_REQUEST: s = "invalid request"; break;
        case MPI_ERR_ROOT: s = "invalid root"; break;
        case MPI_ERR_OP: s = "invalid operation"; break;
        case MPI_ERR_ARG: s = "invalid argument"; break;
        case MPI_ERR_TRUNCATE: s = "message truncated"; break;
        case MPI_ERR_NO_MEM: s = "out of device memory"; break;
        case GPUMPI_ERR_TIMEOUT: s = "device wait timed out"; break;
        case GPUMPI_ERR_ABORTED: s = "job aborted by another rank"; break;
        case GPUMPI_ERR_UNSUPPORTED: s = "unsupported form of call"; break;
        default: break;
    }
    int i = 0;
    for (; s[i] && i < MPI_MAX_ERROR_STRING - 1; i++) string[i] = s[i];
    string[i] = 0;
    *resultlen = i;
    return MPI_SUCCESS;
}

__device__ double MPI_Wtime(void) {
    // %globaltimer is in nanoseconds (the reference scaled clock64 by the SM
    // clock, gpu_libs/gpu_mpi/mpi.cu:142-146).
    return (double)gtime() * 1e-9;
}

__device__ double MPI_Wtick(void) { return 1e-9; }

// ---------------------------------------------------------------- datatypes
__device__ int MPI_Type_size(MPI_Datatype datatype, int* size) {
    int s = dtype_size(datatype);
    if (s < 0) return MPI_ERR_TYPE;
    *size = s;
    return MPI_SUCCESS;
}

__device__ int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype) {
    RankPriv* p = bctx().priv;
    int mult;
    int base = dtype_base(oldtype, &mult);
    if (base < 0) return MPI_ERR_TYPE;
    if (count < 0) return MPI_ERR_COUNT;
    if (p->dt_used >= MAX_DTYPES) return MPI_ERR_INTERN;
    int k = p->dt_used++;
    p->dt_base[k] = base;
    p->dt_count[k] = count * mult;
    *newtype = (MPI_Datatype)(GPUMPI_FIRST_DERIVED_TYPE + k);
    return MPI_SUCCESS;
}

__device__ int MPI_Type_commit(MPI_Datatype* datatype) {
    return dtype_size(*datatype) < 0 ? MPI_ERR_TYPE : MPI_SUCCESS;
}

__device__ int MPI_Type_free(MPI_Datatype* datatype) {
    int t = (int)*datatype;
    if (t >= GPUMPI_FIRST_DERIVED_TYPE) {
        RankPriv* p = bctx().priv;
        int k = t - GPUMPI_FIRST_DERIVED_TYPE;
        if (k < p->dt_used) p->dt_count[k] = -1;
    }
    *datatype = MPI_DATATYPE_NULL;
    return MPI_SUCCESS;
}

__device__ int MPI_Get_count(const MPI_Status* status, MPI_Datatype datatype, int* count) {
    int s = dtype_size(datatype);
    if (s < 0) return MPI_ERR_TYPE;
    u64 bytes = ((u64)(unsigned)status->gpumpi_count_hi << 32) | (unsigned)status->gpumpi_count_lo;
    if (s == 0) {
        *count = 0;
        return MPI_SUCCESS;
    }
    *count = (bytes % s) ? MPI_UNDEFINED : (int)(bytes / s);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- point to point
// A blocking send or receive of an eager message with a basic type, valid
// arguments and no posted receive or deferred send takes the leader-only path
// without a request object (leader_send and recv_small decide by size and
// buffer; a message of at most INLINE_BYTES travels in its header and is sent
// and taken inline here).  Anything else, and a full mailbox, goes through the
// request path, which also reports argument errors.

// The communicator of a leader-path call: context, the caller's rank, size
// and member table (nullptr: ranks are job ranks).  MPI_COMM_WORLD comes from
// the block's cached fields without a memory read, and so does the last other
// communicator used (BlockCtx::sc_*, cleared by MPI_Comm_free).
struct SmallComm {
    int ctx, me, size;
    const int* members;
    __device__ __forceinline__ int job_rank(int r) const { return members ? __ldcg(&members[r]) : r; }
};

// Make `comm` the block's cached communicator; false when it is not a valid
// handle (the request path then reports the error).
static __device__ __noinline__ bool small_comm_cache(MPI_Comm comm) {
    const MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return false;
    BlockCtx& b = bctx();
    b.sc_handle = (const void*)comm;
    b.sc_ctx = c->ctx;
    b.sc_me = c->rank;
    b.sc_size = c->size;
    b.sc_members = c->cs->members;
    return true;
}

// 1: the call may take the leader path (*bytes and *sc set); 0: it takes the
// request path; SMALL_UNCACHED: comm is neither MPI_COMM_WORLD nor the cached
// communicator, and the caller retries after small_comm_cache (through a call
// in tail position, so that nothing stays live across it).
constexpr int SMALL_UNCACHED = -1;
static __device__ __forceinline__ int small_call(const BlockCtx& b, MPI_Comm comm, int count,
                                                 MPI_Datatype datatype, u64* bytes, SmallComm* sc) {
    if (!b.p2p_quiet || count < 0 || (int)datatype < 0 || (int)datatype >= GPUMPI_NUM_BASIC_TYPES) return 0;
    if (comm == &gm_world_sentinel) {
        sc->ctx = b.world_ctx;
        sc->me = b.rank;
        sc->size = b.world_size;
        sc->members = nullptr;
    } else if ((const void*)comm == b.sc_handle) {
        sc->ctx = b.sc_ctx;
        sc->me = b.sc_me;
        sc->size = b.sc_size;
        sc->members = b.sc_members;
    } else {
        return SMALL_UNCACHED;
    }
    *bytes = (u64)count * (u64)basic_size((int)datatype);
    return 1;
}

// Leader: blocking send of a message above INLINE_BYTES without a request
// object (eager up to the eager size, else rendezvous while no lazy receive is
// pending: the blocking rendezvous waits without progressing them, so with
// some pending MPI_Wait on an MPI_Isend request waits instead).  Returns the
// MPI result, or LEADER_PASS when the request path must take the message.  Out of line,
// like the other paths of the blocking calls below, so that the inline path of
// a message of a few bytes saves and restores only the registers it uses.
static __device__ __noinline__ int leader_send_large(const void* buf, u64 bytes, int dj, int ctx, int me, int tag) {
    BlockCtx& b = bctx();
    int rc = MPI_SUCCESS;
    if (bytes <= b.eager_bytes ? p2p_send_small(buf, bytes, dj, ctx, me, tag, &rc)
                               : b.lazy_n == 0 && p2p_send_rdv_small(buf, bytes, dj, ctx, me, tag, &rc))
        return rc;
    return LEADER_PASS;
}

// Leader: blocking eager or rendezvous send; the MPI result, or LEADER_PASS
// when the request path must take the message.
static __device__ __forceinline__ int leader_send(const void* buf, u64 bytes, int dj, int ctx, int me, int tag) {
    if (bytes <= INLINE_BYTES) return send_tiny(buf, (u32)bytes, dj, ctx, me, tag) ? MPI_SUCCESS : LEADER_PASS;
    return leader_send_large(buf, bytes, dj, ctx, me, tag);
}

static __device__ __noinline__ int send_request_path(const void* buf, int count, MPI_Datatype datatype, int dest,
                                                     int tag, MPI_Comm comm) {
    MPI_Request r = MPI_REQUEST_NULL;
    int rc = MPI_Isend(buf, count, datatype, dest, tag, comm, &r);
    if (rc) return rc;
    return MPI_Wait(&r, MPI_STATUS_IGNORE);
}

static __device__ __noinline__ int send_uncached(const void* buf, int count, MPI_Datatype datatype, int dest,
                                                 int tag, MPI_Comm comm) {
    if (!small_comm_cache(comm)) return send_request_path(buf, count, datatype, dest, tag, comm);
    return MPI_Send(buf, count, datatype, dest, tag, comm);
}

static __device__ int start_send(const void* buf, int count, MPI_Datatype datatype, int dest,
                                 int tag, MPI_Comm comm, MPI_Request_impl** out) {
    API_ENTER();
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    int es = dtype_size(datatype);
    if (es < 0) return MPI_ERR_TYPE;
    if (count < 0) return MPI_ERR_COUNT;
    if (tag < 0 || tag > MPI_TAG_UB) return MPI_ERR_TAG;
    if (dest != MPI_PROC_NULL && (dest < 0 || dest >= c->size)) return MPI_ERR_RANK;
    MPI_Request_impl* r = req_alloc();
    if (!r) return MPI_ERR_INTERN;
    const u64 bytes = (u64)count * es;
    r->kind = RK_SEND;
    r->peer = dest;
    r->tag = tag;
    r->ctx = c->ctx;
    r->src_rank = c->rank;
    r->bytes = bytes;
    r->user_buf = (void*)buf;
    r->buf = (void*)buf;
    if (dest == MPI_PROC_NULL) {
        r->state = RS_DONE;
        r->st_source = MPI_PROC_NULL;
        *out = r;
        return MPI_SUCCESS;
    }
    r->peer_world = comm_world_rank(c, dest);
    if (p2p_send_fast(r)) {   // small eager message: the leader alone, straight from buf
        *out = r;
        return MPI_SUCCESS;
    }
    if (p2p_send_rdv_fast(r)) {   // rendezvous from a global buffer, nothing posted on the block path
        *out = r;
        return MPI_SUCCESS;
    }
    if (bytes && !is_global(buf)) {
        void* g = heap_alloc(&b.job->heap, bytes);
        if (!g) {
            req_release(r);
            return MPI_ERR_NO_MEM;
        }
        memcpy(g, buf, bytes);
        r->buf = g;
        r->stage_alloc = 1;
    }
    Call call;
    call.op = OP_SEND_START;
    call.a[0] = (u64)r;
    int rc = block_call(call);
    *out = r;
    return rc;
}

// try_fast (blocking receives): a small eager message that is already or
// soon in the mailbox is taken by the leader alone; otherwise the receive is
// posted on the block path as usual.
static __device__ int start_recv(void* buf, int count, MPI_Datatype datatype, int source, int tag,
                                 MPI_Comm comm, MPI_Request_impl** out, bool try_fast = false) {
    API_ENTER();
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    int es = dtype_size(datatype);
    if (es < 0) return MPI_ERR_TYPE;
    if (count < 0) return MPI_ERR_COUNT;
    if (tag != MPI_ANY_TAG && (tag < 0 || tag > MPI_TAG_UB)) return MPI_ERR_TAG;
    if (source != MPI_PROC_NULL && source != MPI_ANY_SOURCE && (source < 0 || source >= c->size))
        return MPI_ERR_RANK;
    MPI_Request_impl* r = req_alloc();
    if (!r) return MPI_ERR_INTERN;
    const u64 bytes = (u64)count * es;
    r->kind = RK_RECV;
    r->peer = source;
    r->tag = tag;
    r->ctx = c->ctx;
    r->bytes = bytes;
    r->user_buf = buf;
    r->buf = buf;
    if (source == MPI_PROC_NULL) {
        r->state = RS_DONE;
        r->st_source = MPI_PROC_NULL;
        r->st_tag = MPI_ANY_TAG;
        *out = r;
        return MPI_SUCCESS;
    }
    if (try_fast) {
        int handled = 0;
        const int frc = p2p_recv_fast(r, &handled);
        if (frc) {
            req_release(r);
            return frc;
        }
        if (handled) {
            *out = r;
            return MPI_SUCCESS;
        }
    }
    if (bytes && !is_global(buf)) {
        void* g = heap_alloc(&b.job->heap, bytes);
        if (!g) {
            req_release(r);
            return MPI_ERR_NO_MEM;
        }
        r->buf = g;
        r->stage_alloc = 1;
    }
    Call call;
    call.op = OP_RECV_POST;
    call.a[0] = (u64)r;
    int rc = block_call(call);
    *out = r;
    return rc;
}

// Leader: release a completed request, copying staged receive data out.
static __device__ int finish_request(MPI_Request_impl* r, MPI_Status* status) {
    BlockCtx& b = bctx();
    if (r->stage_alloc) {
        if (r->kind == RK_RECV && r->st_bytes) memcpy(r->user_buf, r->buf, r->st_bytes);
        heap_free(&b.job->heap, r->buf);
        r->stage_alloc = 0;
    }
    int err = r->st_err;
    if (r->kind == RK_RECV) fill_status(status, r);
    else if (status) {
        empty_status(status);
    }
    req_release(r);
    return err;
}

__device__ int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag,
                         MPI_Comm comm, MPI_Request* request) {
    MPI_Request_impl* r = nullptr;
    int rc = start_send(buf, count, datatype, dest, tag, comm, &r);
    *request = r;
    return rc;
}

__device__ int MPI_Irecv(void* buf, int count, MPI_Datatype datatype, int source, int tag,
                         MPI_Comm comm, MPI_Request* request) {
    {
        // a lazy receive: matched by the leader when it is waited for (lazy_progress)
        BlockCtx& b = bctx();
        u64 bytes;
        SmallComm sc;
        int k = b.lazy_n < LAZY_MAX ? small_call(b, comm, count, datatype, &bytes, &sc) : 0;
        if (k == SMALL_UNCACHED) k = small_comm_cache(comm) ? small_call(b, comm, count, datatype, &bytes, &sc) : 0;
        if (k == 1 &&
            (source == MPI_ANY_SOURCE || (source >= 0 && source < sc.size)) &&
            (tag == MPI_ANY_TAG || (tag >= 0 && tag <= MPI_TAG_UB))) {
            if (api_abort_check(b)) return aborted_code();
            MPI_Request_impl* r = req_alloc();
            if (r) {
                r->kind = RK_RECV;
                r->peer = source;
                r->tag = tag;
                r->ctx = sc.ctx;
                r->bytes = bytes;
                r->user_buf = buf;
                r->buf = buf;
                r->state = RS_LAZY;
                b.lazy[b.lazy_n++] = r->index;
                *request = r;
                return MPI_SUCCESS;
            }
        }
    }
    MPI_Request_impl* r = nullptr;
    int rc = start_recv(buf, count, datatype, source, tag, comm, &r);
    *request = r;
    return rc;
}

__device__ int MPI_Wait(MPI_Request* request, MPI_Status* status) {
    API_ENTER();
    if (!request || *request == MPI_REQUEST_NULL) {
        empty_status(status);
        return MPI_SUCCESS;
    }
    MPI_Request_impl* r = *request;
    if (!req_valid(r)) return MPI_ERR_REQUEST;
    if (r->state == RS_LAZY) {
        const int rc = lazy_wait(r);   // done, or posted on the block path
        if (rc) return rc;
    }
    if (r->state == RS_WAIT_RDV && b.p2p_quiet) {
        const int rc = rdv_wait_leader(r);   // done, or the block path takes over
        if (rc) return rc;
    }
    if (r->state != RS_DONE) {
        Call call;
        call.op = OP_WAIT;
        call.a[0] = (u64)r;
        int rc = block_call(call);
        if (rc) return rc;
    }
    *request = MPI_REQUEST_NULL;
    return finish_request(r, status);
}

__device__ int MPI_Test(MPI_Request* request, int* flag, MPI_Status* status) {
    API_ENTER();
    if (!request || *request == MPI_REQUEST_NULL) {
        *flag = 1;
        empty_status(status);
        return MPI_SUCCESS;
    }
    MPI_Request_impl* r = *request;
    if (!req_valid(r)) return MPI_ERR_REQUEST;
    if (r->state == RS_LAZY) {
        const int rc = lazy_progress();
        if (rc) return rc;
        if (r->state == RS_LAZY) {
            *flag = 0;
            return MPI_SUCCESS;
        }
    }
    int done = r->state == RS_DONE;
    if (!done) {
        Call call;
        call.op = OP_TEST;
        call.a[0] = (u64)r;
        int rc = block_call(call);
        if (rc) return rc;
        done = (int)call.a[1];
    }
    *flag = done;
    if (!done) return MPI_SUCCESS;
    *request = MPI_REQUEST_NULL;
    return finish_request(r, status);
}

__device__ int MPI_Waitall(int count, MPI_Request array_of_requests[], MPI_Status* array_of_statuses) {
    int first = MPI_SUCCESS;
    for (int i = 0; i < count; i++) {
        int rc = MPI_Wait(&array_of_requests[i],
                          array_of_statuses ? &array_of_statuses[i] : MPI_STATUS_IGNORE);
        if (rc && !first) first = rc;
    }
    return first;
}

__device__ int MPI_Testall(int count, MPI_Request array_of_requests[], int* flag,
                           MPI_Status array_of_statuses[]) {
    API_ENTER();
    int all = 1;
    for (int i = 0; i < count; i++) {
        MPI_Request_impl* r = array_of_requests[i];
        if (r == MPI_REQUEST_NULL) continue;
        if (!req_valid(r)) return MPI_ERR_REQUEST;
        if (r->state != RS_DONE) {
            Call call;
            call.op = OP_TEST;
            call.a[0] = (u64)r;
            int rc = block_call(call);
            if (rc) return rc;
            if (!call.a[1]) all = 0;
        }
    }
    *flag = all;
    if (!all) return MPI_SUCCESS;
    int first = MPI_SUCCESS;
    for (int i = 0; i < count; i++) {
        MPI_Request_impl* r = array_of_requests[i];
        MPI_Status* st = array_of_statuses ? &array_of_statuses[i] : MPI_STATUS_IGNORE;
        if (r == MPI_REQUEST_NULL) {
            empty_status(st);
            continue;
        }
        array_of_requests[i] = MPI_REQUEST_NULL;
        int rc = finish_request(r, st);
        if (rc && !first) first = rc;
    }
    return first;
}

__device__ int MPI_Waitany(int count, MPI_Request array_of_requests[], int* index,
                           MPI_Status* status) {
    API_ENTER();
    const u64 t0 = gtime();
    for (;;) {
        int active = 0;
        for (int i = 0; i < count; i++) {
            MPI_Request_impl* r = array_of_requests[i];
            if (r == MPI_REQUEST_NULL) continue;
            if (!req_valid(r)) return MPI_ERR_REQUEST;
            active = 1;
            int done = r->state == RS_DONE;
            if (!done) {
                Call call;
                call.op = OP_TEST;
                call.a[0] = (u64)r;
                int rc = block_call(call);
                if (rc) return rc;
                done = (int)call.a[1];
            }
            if (done) {
                *index = i;
                array_of_requests[i] = MPI_REQUEST_NULL;
                return finish_request(r, status);
            }
        }
        if (!active) {
            *index = MPI_UNDEFINED;
            empty_status(status);
            return MPI_SUCCESS;
        }
        if (job_aborted(b.job)) return aborted_code();
        if (gtime() - t0 > b.job->timeout_ns) {
            job_fail(b.job, b.rank, GPUMPI_ERR_TIMEOUT, "MPI_Waitany timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(128);
    }
}

__device__ int MPI_Waitsome(int incount, MPI_Request array_of_requests[], int* outcount,
                            int array_of_indices[], MPI_Status array_of_statuses[]) {
    API_ENTER();
    const u64 t0 = gtime();
    for (;;) {
        int active = 0, n = 0;
        for (int i = 0; i < incount; i++) {
            MPI_Request_impl* r = array_of_requests[i];
            if (r == MPI_REQUEST_NULL) continue;
            if (!req_valid(r)) return MPI_ERR_REQUEST;
            active = 1;
            int done = r->state == RS_DONE;
            if (!done) {
                Call call;
                call.op = OP_TEST;
                call.a[0] = (u64)r;
                int rc = block_call(call);
                if (rc) return rc;
                done = (int)call.a[1];
            }
            if (done) {
                array_of_indices[n] = i;
                array_of_requests[i] = MPI_REQUEST_NULL;
                finish_request(r, array_of_statuses ? &array_of_statuses[n] : MPI_STATUS_IGNORE);
                n++;
            }
        }
        if (!active) {
            *outcount = MPI_UNDEFINED;
            return MPI_SUCCESS;
        }
        if (n > 0) {
            *outcount = n;
            return MPI_SUCCESS;
        }
        if (job_aborted(b.job)) return aborted_code();
        if (gtime() - t0 > b.job->timeout_ns) {
            job_fail(b.job, b.rank, GPUMPI_ERR_TIMEOUT, "MPI_Waitsome timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(128);
    }
}

__device__ int MPI_Request_free(MPI_Request* request) {
    if (!request || *request == MPI_REQUEST_NULL) return MPI_SUCCESS;
    MPI_Request_impl* r = *request;
    if (!req_valid(r)) return MPI_ERR_REQUEST;
    // An active request must still complete; wait for it so its buffers stay valid.
    int rc = MPI_SUCCESS;
    if (r->state != RS_DONE) {
        Call call;
        call.op = OP_WAIT;
        call.a[0] = (u64)r;
        rc = block_call(call);
        if (rc) return rc;
    }
    *request = MPI_REQUEST_NULL;
    finish_request(r, MPI_STATUS_IGNORE);
    return rc;
}


__device__ int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int dest, int tag,
                        MPI_Comm comm) {
    BlockCtx& b = bctx();
    u64 bytes;
    SmallComm sc;
    const int k = small_call(b, comm, count, datatype, &bytes, &sc);
    if (k == SMALL_UNCACHED) return send_uncached(buf, count, datatype, dest, tag, comm);
    if (k && dest >= 0 && dest < sc.size && tag >= 0 && tag <= MPI_TAG_UB) {
        if (api_abort_check(b)) return aborted_code();
        const int rc = leader_send(buf, bytes, sc.job_rank(dest), sc.ctx, sc.me, tag);
        if (rc != LEADER_PASS) return rc;
    }
    return send_request_path(buf, count, datatype, dest, tag, comm);
}

__device__ int MPI_Ssend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag,
                         MPI_Comm comm) {
    return MPI_Send(buf, count, datatype, dest, tag, comm);
}

static __device__ __noinline__ int recv_request_path(void* buf, int count, MPI_Datatype datatype, int source,
                                                     int tag, MPI_Comm comm, MPI_Status* status) {
    MPI_Request r = MPI_REQUEST_NULL;
    int rc = start_recv(buf, count, datatype, source, tag, comm, &r, /*try_fast=*/true);
    if (rc) return rc;
    return MPI_Wait(&r, status);
}

static __device__ __noinline__ int recv_uncached(void* buf, int count, MPI_Datatype datatype, int source, int tag,
                                                 MPI_Comm comm, MPI_Status* status) {
    if (!small_comm_cache(comm)) return recv_request_path(buf, count, datatype, source, tag, comm, status);
    return MPI_Recv(buf, count, datatype, source, tag, comm, status);
}

__device__ int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int source, int tag,
                        MPI_Comm comm, MPI_Status* status) {
    BlockCtx& b = bctx();
    u64 bytes;
    SmallComm sc;
    const int k = b.lazy_n == 0 ? small_call(b, comm, count, datatype, &bytes, &sc) : 0;
    if (k == SMALL_UNCACHED) return recv_uncached(buf, count, datatype, source, tag, comm, status);
    if (k && (source == MPI_ANY_SOURCE || (source >= 0 && source < sc.size)) &&
        (tag == MPI_ANY_TAG || (tag >= 0 && tag <= MPI_TAG_UB))) {
        if (api_abort_check(b)) return aborted_code();
        const int rc = recv_small(buf, bytes, sc.ctx, source, tag, status);
        if (rc != LEADER_PASS) return rc;
    }
    return recv_request_path(buf, count, datatype, source, tag, comm, status);
}

// A real exchange; the reference's version was an empty stub (gpu_libs/gpu_mpi/mpi.cu:255-260).
__device__ int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest,
                            int sendtag, void* recvbuf, int recvcount, MPI_Datatype recvtype,
                            int source, int recvtag, MPI_Comm comm, MPI_Status* status) {
    {
        // An eager send completes without the receiver, so the leader may send
        // first and then receive (the halo exchanges of stencil codes).
        BlockCtx& b = bctx();
        u64 sbytes;
        SmallComm sc;
        int k = small_call(b, comm, sendcount, sendtype, &sbytes, &sc);
        if (k == SMALL_UNCACHED) k = small_comm_cache(comm) ? small_call(b, comm, sendcount, sendtype, &sbytes, &sc) : 0;
        if (k == 1 && sbytes <= b.eager_bytes &&
            recvcount >= 0 && (int)recvtype >= 0 && (int)recvtype < GPUMPI_NUM_BASIC_TYPES && dest >= 0 &&
            dest < sc.size && sendtag >= 0 && sendtag <= MPI_TAG_UB &&
            (source == MPI_ANY_SOURCE || (source >= 0 && source < sc.size)) &&
            (recvtag == MPI_ANY_TAG || (recvtag >= 0 && recvtag <= MPI_TAG_UB))) {
            if (api_abort_check(b)) return aborted_code();
            const int rc = leader_send(sendbuf, sbytes, sc.job_rank(dest), sc.ctx, sc.me, sendtag);
            if (rc != LEADER_PASS) return rc ? rc : MPI_Recv(recvbuf, recvcount, recvtype, source, recvtag, comm, status);
        }
    }
    MPI_Request rr = MPI_REQUEST_NULL, sr = MPI_REQUEST_NULL;
    int rc = MPI_Irecv(recvbuf, recvcount, recvtype, source, recvtag, comm, &rr);
    if (rc) return rc;
    rc = MPI_Isend(sendbuf, sendcount, sendtype, dest, sendtag, comm, &sr);
    if (rc) return rc;
    int rc1 = MPI_Wait(&sr, MPI_STATUS_IGNORE);
    int rc2 = MPI_Wait(&rr, status);
    return rc1 ? rc1 : rc2;
}

__device__ int MPI_Sendrecv_replace(void* buf, int count, MPI_Datatype datatype, int dest,
                                    int sendtag, int source, int recvtag, MPI_Comm comm,
                                    MPI_Status* status) {
    API_ENTER();
    int es = dtype_size(datatype);
    if (es < 0) return MPI_ERR_TYPE;
    u64 bytes = (u64)count * es;
    void* tmp = bytes ? heap_alloc(&b.job->heap, bytes) : nullptr;
    if (bytes && !tmp) return MPI_ERR_NO_MEM;
    if (bytes) memcpy(tmp, buf, bytes);
    int rc = MPI_Sendrecv(tmp, count, datatype, dest, sendtag, buf, count, datatype, source,
                          recvtag, comm, status);
    if (tmp) heap_free(&b.job->heap, tmp);
    return rc;
}

static __device__ int probe_common(int source, int tag, MPI_Comm comm, int blocking, int* flag,
                                   MPI_Status* status) {
    API_ENTER();
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    if (source == MPI_PROC_NULL) {
        if (flag) *flag = 1;
        if (status) {
            empty_status(status);
            status->MPI_SOURCE = MPI_PROC_NULL;
        }
        return MPI_SUCCESS;
    }
    MPI_Status local;
    Call call;
    call.op = OP_PROBE;
    call.a[0] = (u64)&local;
    call.a[2] = (u64)(long long)source;
    call.a[3] = (u64)(long long)tag;
    call.a[4] = (u64)c->ctx;
    call.a[5] = (u64)blocking;
    int rc = block_call(call);
    if (rc) return rc;
    if (flag) *flag = (int)call.a[1];
    if (call.a[1] && status) *status = local;
    return MPI_SUCCESS;
}

__device__ int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* status) {
    return probe_common(source, tag, comm, 0, flag, status);
}

__device__ int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* status) {
    return probe_common(source, tag, comm, 1, nullptr, status);
}
