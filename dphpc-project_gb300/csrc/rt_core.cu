// Core of the device runtime: handle sentinels, job status and bounded waits,
// the block-cooperative copy engine, the leader/helper call protocol and the
// per-rank lifecycle.
#include "rt.cuh"

// ---------------------------------------------------------------- sentinels
// MPI_COMM_WORLD / MPI_COMM_SELF / MPI_GROUP_WORLD / MPI_GROUP_EMPTY are the
// addresses of these objects; every rank resolves them to its own job.
__device__ MPI_Comm_impl gm_world_sentinel = {2, 0, 0, 0, 0, 0, nullptr, 0};
__device__ MPI_Comm_impl gm_self_sentinel = {3, 0, 0, 0, 0, 0, nullptr, 0};
__device__ MPI_Group_impl gm_group_world_sentinel = {2, 0, nullptr, 0, 0};
__device__ MPI_Group_impl gm_group_empty_sentinel = {3, 0, nullptr, 0, 0};

__device__ MPI_Comm MPI_COMM_WORLD = &gm_world_sentinel;
__device__ MPI_Comm MPI_COMM_SELF = &gm_self_sentinel;
__device__ MPI_Comm MPI_COMM_NULL = nullptr;
__device__ MPI_Group MPI_GROUP_WORLD = &gm_group_world_sentinel;
__device__ MPI_Group MPI_GROUP_EMPTY = &gm_group_empty_sentinel;
__device__ MPI_Group MPI_GROUP_NULL = nullptr;

namespace gm {

// ---------------------------------------------------------------- job status
__device__ void job_fail(Job* j, int rank, int code, const char* msg) {
    if (atomicCAS(&j->status[1], 0, code) == 0) {
        j->status[2] = rank;
        int i = 0;
        if (msg) {
            for (; i < 255 && msg[i]; i++) j->err_msg[i] = msg[i];
        }
        j->err_msg[i] = 0;
    }
    __threadfence();
    atomicExch(&j->status[0], 1);
}

// Code returned by a wait that ended because the job failed: the rank that
// recorded the job's first error gets that error (e.g. its own timeout); every
// rank released by another rank's failure gets GPUMPI_ERR_ABORTED.
__device__ int fail_code(Job* j) {
    const int code = ld_acquire_int(&j->status[1]);
    if (code && ld_acquire_int(&j->status[2]) == bctx().rank) return code;
    return GPUMPI_ERR_ABORTED;
}

static __device__ __forceinline__ int wait_fail(Job* j) { return fail_code(j); }

__device__ int wait_ge(const u64* addr, u64 target) {
    if (ld_acquire(addr) >= target) return MPI_SUCCESS;
    Job* j = bctx().job;
    u64 t0 = gtime();
    unsigned ns = 32;
    for (;;) {
        if (ld_acquire(addr) >= target) return MPI_SUCCESS;
        if (job_aborted(j)) return wait_fail(j);
        if (gtime() - t0 > j->timeout_ns) {
            job_fail(j, bctx().rank, GPUMPI_ERR_TIMEOUT, "collective wait timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
    }
}

__device__ int wait_u32_nonzero(const volatile u32* addr) {
    if (*addr) return MPI_SUCCESS;
    Job* j = bctx().job;
    u64 t0 = gtime();
    unsigned ns = 32;
    for (;;) {
        if (ld_acquire32((const u32*)addr)) return MPI_SUCCESS;
        if (job_aborted(j)) return wait_fail(j);
        if (gtime() - t0 > j->timeout_ns) {
            job_fail(j, bctx().rank, GPUMPI_ERR_TIMEOUT, "point-to-point wait timed out");
            return GPUMPI_ERR_TIMEOUT;
        }
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
    }
}

// All threads of the block poll a slice of `flags` (every entry except `skip`)
// until each is >= target.  Returns the same code on every thread.
__device__ int wait_flags_ge(const u64* flags, int n, u64 target, int skip, int tid, int T) {
    int rc = MPI_SUCCESS;
    for (int q = tid; q < n; q += T) {
        if (q == skip) continue;
        rc = wait_ge(&flags[q], target);
        if (rc) break;
    }
    int failed = bar_or(rc != MPI_SUCCESS, T);
    if (!failed) return MPI_SUCCESS;
    return wait_fail(bctx().job);
}

// ---------------------------------------------------------------- copies
// Each thread copies vectors tid, tid + T, ... with U loads in flight, the last
// partial batch included: a copy of a few vectors per thread (a 2-KiB block
// copied by one warp) then waits one memory round trip, not one per vector.
template <class V, int U>
static __device__ __forceinline__ void copy_vec(V* __restrict__ d, const V* __restrict__ s, u64 nv,
                                                u64 tid, u64 T) {
    u64 i = tid;
    for (; i + (U - 1) * T < nv; i += U * T) {
        V r[U];
#pragma unroll
        for (int k = 0; k < U; k++) r[k] = __ldcg(s + i + k * T);
#pragma unroll
        for (int k = 0; k < U; k++) d[i + k * T] = r[k];
    }
    if (i < nv) {
        V r[U];
#pragma unroll
        for (int k = 0; k < U; k++)
            if (i + k * T < nv) r[k] = __ldcg(s + i + k * T);
#pragma unroll
        for (int k = 0; k < U; k++)
            if (i + k * T < nv) d[i + k * T] = r[k];
    }
}

static __device__ __forceinline__ void copy_range(char* d, const char* s, u64 n, u64 tid, u64 T) {
    uintptr_t da = (uintptr_t)d, sa = (uintptr_t)s;
    if (((da ^ sa) & 15) == 0) {
        u64 head = (16 - (da & 15)) & 15;
        if (head > n) head = n;
        for (u64 i = tid; i < head; i += T) d[i] = __ldcg(s + i);
        d += head;
        s += head;
        n -= head;
        u64 nv = n >> 4;
        copy_vec<uint4, 8>((uint4*)d, (const uint4*)s, nv, tid, T);
        u64 done = nv << 4;
        for (u64 i = done + tid; i < n; i += T) d[i] = __ldcg(s + i);
    } else if (((da ^ sa) & 7) == 0) {
        u64 head = (8 - (da & 7)) & 7;
        if (head > n) head = n;
        for (u64 i = tid; i < head; i += T) d[i] = __ldcg(s + i);
        d += head;
        s += head;
        n -= head;
        u64 nv = n >> 3;
        copy_vec<uint2, 8>((uint2*)d, (const uint2*)s, nv, tid, T);
        u64 done = nv << 3;
        for (u64 i = done + tid; i < n; i += T) d[i] = __ldcg(s + i);
    } else if (((da ^ sa) & 3) == 0) {
        u64 head = (4 - (da & 3)) & 3;
        if (head > n) head = n;
        for (u64 i = tid; i < head; i += T) d[i] = __ldcg(s + i);
        d += head;
        s += head;
        n -= head;
        u64 nv = n >> 2;
        copy_vec<unsigned int, 8>((unsigned int*)d, (const unsigned int*)s, nv, tid, T);
        u64 done = nv << 2;
        for (u64 i = done + tid; i < n; i += T) d[i] = __ldcg(s + i);
    } else {
        for (u64 i = tid; i < n; i += T) d[i] = __ldcg(s + i);
    }
}

// ---------------------------------------------------------------- bulk engine
static __device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ u32 bulk_stage_bytes() {
    u32 dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    // a one-cluster job keeps its mailbox at the end of dynamic shared memory
    const u32 base = BCTX_BYTES + BULK_BAR_BYTES + (bctx().mb_cluster ? (u32)MB_SMEM_BYTES : 0u);
    return dyn > base ? dyn - base : 0;
}

__device__ bool BulkPipe::begin() {
    const u32 bytes = bulk_stage_bytes();
    chunk = (bytes / BULK_STAGES) & ~15u;
    if (chunk < 2048 || bctx().bulk_broken) return false;
    extern __shared__ __align__(16) char gm_dsmem[];
    bars = reinterpret_cast<u64*>(gm_dsmem + BCTX_BYTES);
    stage = gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES;
    issued = stored = 0;
    err = 0;
    for (int s = 0; s < BULK_STAGES; s++)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[s])) : "memory");
    // the barriers are used by the async proxy; data the bulk loads read was
    // written (and acquired) through the generic proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
    return true;
}

// Wait for the oldest loaded chunk and start its store.
__device__ bool BulkPipe::retire() {
    const int s = (int)(stored % BULK_STAGES);
    const u32 parity = (u32)((stored / BULK_STAGES) & 1);
    const u32 bar = smem_u32(&bars[s]);
    u32 done = 0;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                 : "=r"(done) : "r"(bar), "r"(parity) : "memory");
    if (!done) {
        Job* j = bctx().job;
        const u64 t0 = gtime();
        while (!done) {
            asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                         : "=r"(done) : "r"(bar), "r"(parity) : "memory");
            if (!done && gtime() - t0 > j->timeout_ns) {
                job_fail(j, bctx().rank, GPUMPI_ERR_TIMEOUT, "bulk copy did not complete");
                err = GPUMPI_ERR_TIMEOUT;
                return false;
            }
        }
    }
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                 ::"l"(dst_of[s]), "r"(smem_u32(stage + (u64)s * chunk)), "r"(len_of[s]) : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    stored++;
    return true;
}

// Schedule: at most BULK_STAGES - 1 loads wait; before a load reuses a stage,
// the oldest load is retired (its store issued) and only the store issued one
// step earlier, which used this stage, must have finished reading it; the
// newest store may still be reading its own stage.
__device__ bool BulkPipe::push(char* dst, const char* src, u64 n) {
    while (n > 0 && !err) {
        const u32 len = n < chunk ? (u32)n : chunk;
        if (issued - stored == BULK_STAGES - 1 && !retire()) return false;
        // the stage is free once the store that last used it (#issued - BULK_STAGES) has read it;
        // stores newer than that one may stay in flight
        if (issued >= BULK_STAGES) {
            if (stored - (issued - BULK_STAGES) >= 2)
                asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
            else
                asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
        const int s = (int)(issued % BULK_STAGES);
        const u32 bar = smem_u32(&bars[s]);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(len) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(smem_u32(stage + (u64)s * chunk)), "l"(src), "r"(len), "r"(bar) : "memory");
        dst_of[s] = dst;
        len_of[s] = len;
        issued++;
        dst += len;
        src += len;
        n -= len;
    }
    return !err;
}

__device__ int BulkPipe::finish() {
    while (stored < issued && retire()) {
    }
    // The stores issued so far are waited for in every case.
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    asm volatile("fence.proxy.async.global;" ::: "memory");
    if (err) {
        // loads may still be in flight: the barriers stay as they are and this
        // block copies with vector loads from now on
        bctx().bulk_broken = 1;
        return err;
    }
    // every load completed: retire the barriers, so that the next pipeline may
    // initialise this memory again (mbarrier.init on a live barrier is undefined)
    for (int s = 0; s < BULK_STAGES; s++)
        asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(&bars[s])) : "memory");
    return err;
}

// Large aligned copies go through the bulk engine, driven by thread 0 (the
// other threads only copy the unaligned tail); the block synchronises after.
__device__ void blk_copy(void* dst, const void* src, u64 n, int tid, int T) {
    if (n == 0 || dst == src) return;
    if (n >= BULK_MIN_BYTES && (((uintptr_t)dst | (uintptr_t)src) & 15) == 0 && bulk_stage_bytes() >= 8192 &&
        bctx().job != nullptr) {
        const u64 n16 = n & ~(u64)15;
        if (tid == 0) {
            BulkPipe bp;
            if (bp.begin()) {
                bp.push((char*)dst, (const char*)src, n16);
                bp.finish();
            } else {
                copy_range((char*)dst, (const char*)src, n16, 0, 1);
            }
        }
        if (n16 < n) copy_range((char*)dst + n16, (const char*)src + n16, n - n16, (u64)tid, (u64)T);
        bsync();
        return;
    }
    copy_range((char*)dst, (const char*)src, n, (u64)tid, (u64)T);
}

__device__ void warp_copy(void* dst, const void* src, u64 n, int lane) {
    if (n == 0 || dst == src) return;
    copy_range((char*)dst, (const char*)src, n, (u64)lane, 32);
}

__device__ void blk_memset(void* dst, int c, u64 n, int tid, int T) {
    char* d = (char*)dst;
    unsigned char b = (unsigned char)c;
    uintptr_t da = (uintptr_t)d;
    u64 head = (16 - (da & 15)) & 15;
    if (head > n) head = n;
    for (u64 i = tid; i < head; i += T) d[i] = b;
    d += head;
    n -= head;
    u64 nv = n >> 4;
    unsigned w = b * 0x01010101u;
    uint4 v = make_uint4(w, w, w, w);
    uint4* dv = (uint4*)d;
    for (u64 i = tid; i < nv; i += T) dv[i] = v;
    for (u64 i = (nv << 4) + tid; i < n; i += T) d[i] = b;
}

// ---------------------------------------------------------------- call protocol
__device__ int block_call(Call& c) {
    BlockCtx& b = bctx();
    mb_release_taken();   // the block path may wait on senders that need those slots
    // Lazy receives go to the block path before any point-to-point call there:
    // it matches in posting order, and a wait on a rendezvous send needs the
    // receives it depends on to progress (two ranks in MPI_Sendrecv).
    if (b.lazy_n > 0 &&
        (c.op == OP_SEND_START || c.op == OP_RECV_POST || c.op == OP_WAIT || c.op == OP_TEST ||
         c.op == OP_PROBE || c.op == OP_FINALIZE)) {
        const int rc = lazy_materialize();
        if (rc) return rc;
    }
    b.call = c;
    b.in_call = 1;
    bar_named(1, b.T);
    int rc = dispatch_all(0);
    bar_named(1, b.T);
    b.in_call = 0;
    c = b.call;
    return rc;
}

__device__ void helper_loop() {
    BlockCtx& b = bctx();
    const int tid = threadIdx.x;
    for (;;) {
        bar_named(1, b.T);
        if (b.call.op == OP_EXIT) break;
        dispatch_all(tid);
        bar_named(1, b.T);
    }
}

// ---------------------------------------------------------------- staging
__device__ void* stage_temp(int bytes) {
    RankPriv* p = bctx().priv;
    int off = (p->stage_off + 15) & ~15;
    if (off + bytes > STAGE_BYTES) return nullptr;
    p->stage_off = off + bytes;
    return p->stage + off;
}
__device__ void stage_reset() { bctx().priv->stage_off = 0; }

// ---------------------------------------------------------------- handles
__device__ MPI_Comm_impl* comm_resolve(MPI_Comm c) {
    RankPriv* p = bctx().priv;
    if (c == &gm_world_sentinel) return &p->comms[0];
    if (c == &gm_self_sentinel) return &p->comms[1];
    if (c == nullptr) return nullptr;
    if (c < &p->comms[0] || c >= &p->comms[MAX_COMMS]) return nullptr;
    if (c->kind != 1) return nullptr;
    return c;
}

// ---------------------------------------------------------------- output
__device__ int out_write(Job* j, int stream, const char* s, int n) {
    if (n <= 0) return 0;
    char* buf = stream == 2 ? j->errout : j->out;
    u64* offp = stream == 2 ? j->errout_off : j->out_off;
    u64 off = atomicAdd(offp, (u64)n);
    if (off >= j->out_bytes) return 0;
    u64 m = n;
    if (off + m > j->out_bytes) m = j->out_bytes - off;
    for (u64 i = 0; i < m; i++) buf[off + i] = s[i];
    return (int)m;
}

// ---------------------------------------------------------------- lifecycle
__device__ void rank_init(int tid, int T) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    RankPriv* p = b.priv;
    const int r = b.rank;
    MPI_Request_impl* reqs = j->reqpool + (u64)r * j->max_requests;
    // Rank-private state is written and read by thread 0 only.
    if (tid == 0) {
        for (int i = 0; i < j->max_requests; i++) {
            reqs[i].kind = RK_FREE;
            reqs[i].state = RS_NEW;
            reqs[i].index = i;
            reqs[i].next = (i + 1 < j->max_requests) ? i + 1 : -1;
        }
        for (int i = 0; i < MAX_COMMS; i++) p->comms[i].kind = 0;
        for (int i = 0; i < MAX_GROUPS; i++) p->groups[i].kind = 0;
        p->reqs = reqs;
        p->nreqs = j->max_requests;
        p->free_head = j->max_requests > 0 ? 0 : -1;
        p->recv_head = p->recv_tail = -1;
        p->defer_head = p->defer_tail = -1;
        p->initialized = 0;
        p->finalized = 0;
        p->errno_v = 0;
        p->opt_ind = 1;
        p->opt_err = 1;
        p->opt_opt = 0;
        p->opt_pos = 0;
        p->opt_arg = nullptr;
        p->strtok_save = nullptr;
        p->rng = 0x9E3779B97F4A7C15ull ^ ((u64)r * 0xD1B54A32D192ED03ull);
        p->stage = j->stage + (u64)r * STAGE_BYTES;
        p->stage_off = 0;
        p->exited = 0;
        p->dt_used = 0;
        MPI_Comm_impl& w = p->comms[0];
        w.kind = 1;
        w.ctx = 1;
        w.size = j->nranks;
        b.mbox = j->mbox;
        b.eager = j->eager;
        b.eager_bytes = j->eager_bytes;
        b.timeout_ns = j->timeout_ns;
        b.slot_hint = 0;
        b.world_ctx = 1;
        b.world_size = j->nranks;
        b.p2p_quiet = 1;
        b.api_calls = 0;
        b.lazy_n = 0;
        b.sc_handle = nullptr;
        w.rank = r;
        w.refcnt = 1;
        w.cs = j->world_cs;
        w.seq = 0;
        MPI_Comm_impl& s = p->comms[1];
        s.kind = 1;
        s.ctx = 2;
        s.size = 1;
        s.rank = 0;
        s.refcnt = 1;
        s.cs = &j->self_cs[r];
        s.seq = 0;
    }
    __syncthreads();
}

// End the calling rank from the leader thread: record the status, release the
// helper threads (they leave the kernel) and retire the leader with PTX `exit`.
__device__ void rank_exit_now(int status) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    b.priv->exited = 1;
    if (status != 0) {
        atomicCAS(&j->status[6], 0, status);
        job_fail(j, b.rank, GPUMPI_ERR_ABORTED, "a rank called exit() or abort() with nonzero status");
    }
    cluster_release();
    rank_finish(status);
    if (b.leader_mode && !b.in_call) {
        b.call.op = OP_EXIT;
        bar_named(1, b.T);
    }
    asm volatile("exit;");
}

__device__ void rank_finish(int rc) {
    BlockCtx& b = bctx();
    Job* j = b.job;
    j->retvals[b.rank] = rc;
    __threadfence();
    atomicAdd(&j->status[3], 1);
}

}  // namespace gm

namespace gm {

// Thread 0: the block context of rank `rank` of `job` in rank slot `slot`,
// block `crank` of a rank made of C blocks.
static __device__ void block_ctx_init(Job* job, int rank, int slot, u32 C, u32 crank) {
    BlockCtx& b = bctx();
    b.job = job;
    b.rank = rank;
    b.priv = &job->priv[rank];
    b.slot = slot;
    b.T = (int)blockDim.x;
    b.leader_mode = 1;
    b.in_call = 0;
    b.bulk_broken = 0;
    b.lazy_n = 0;
    b.mb_taken = 0;
    b.call.op = -1;
    b.cl_n = (int)C;
    b.cl_rank = (int)crank;
    b.cl_released = 0;
    b.cl_phase = 0;
    b.cl_cmd.op = -1;
    b.mb_cluster = 0;
    b.mb_local = nullptr;
    if (crank > 0) b.leader_mode = 0;   // a helper block of a cluster rank
}

// Worker blocks of a server: one rank of one block, set up and initialised.
__device__ void rank_block_setup(Job* job, int rank, int slot) {
    if (threadIdx.x == 0) block_ctx_init(job, rank, slot, 1, 0);
    __syncthreads();
    rank_init((int)threadIdx.x, (int)blockDim.x);
}

// Block set-up for program kernels: find this slot's job and rank, then
// initialise the rank.  Returns false for idle slots.
__device__ bool program_block_begin(const Launch& L) {
    BlockCtx& b = bctx();
    // a rank is one cluster: C consecutive blocks (C = 1 without a cluster
    // launch, and for a job that is one cluster of one-block ranks)
    u32 C, crank;
    asm("mov.u32 %0, %%cluster_nctarank;" : "=r"(C));
    asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(crank));
    const u32 launch_cluster = C;   // blocks in this launch's clusters
    if (L.job_cluster) {
        C = 1;
        crank = 0;
    }
    const int slot = (int)(blockIdx.x / C);
    if (threadIdx.x == 0) {
        const int jid = slot < L.nslots ? L.slot_job[slot] : -1;
        if (jid < 0) {
            b.job = nullptr;
        } else {
            block_ctx_init(&L.jobs[jid], L.slot_rank[slot], L.slot_base + slot, C, crank);
            // mailboxes in shared memory only when the launch really made the
            // job's ranks one cluster (the same answer in every block of the
            // launch); otherwise the ranks keep their mailboxes in HBM, which
            // every job has, instead of addressing blocks outside their cluster
            if (L.job_cluster && launch_cluster == (u32)L.jobs[jid].nranks) {
                extern __shared__ __align__(16) char gm_dsmem[];
                u32 dyn;
                asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
                b.mb_cluster = 1;
                b.mb_local = reinterpret_cast<Mailbox*>(gm_dsmem + ((dyn - (u32)MB_SMEM_BYTES) & ~127u));
            }
        }
    }
    __syncthreads();
    if (L.job_cluster) {
        // every block clears its mailbox before any block may write to it
        if (b.job && b.mb_cluster) blk_memset(b.mb_local, 0, sizeof(Mailbox), (int)threadIdx.x, (int)blockDim.x);
        asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
    }
    if (!b.job) return false;
    if (crank == 0) rank_init((int)threadIdx.x, (int)blockDim.x);
    cluster_setup((int)threadIdx.x);
    return true;
}

// End of a block of a one-cluster job: its shared memory holds its rank's
// mailbox, which the other ranks' blocks may address until every block is
// done, so no block leaves before all have arrived here (threads that left
// the kernel early, such as a leader that called exit(), do not count).
__device__ void program_block_end(const Launch& L) {
    if (L.job_cluster) asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}


}  // namespace gm
