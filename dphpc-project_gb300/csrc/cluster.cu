// Ranks as thread-block clusters.
//
// A job launched with C > 1 blocks per rank runs every rank as one cluster of
// C thread blocks (C = 2, 4 or 8, on up to C SMs).  Block 0 of the cluster is
// the rank block of the one-block model: its thread 0 runs the converted
// program and its other threads execute the rank's MPI calls.  Blocks 1..C-1
// ("helper blocks") take shares of the rank's parallel loops
// (gpumpi_parallel_for), so a job with fewer ranks than SMs computes on C
// times as many SMs.  This extends the reference's launch, where a rank was
// one thread (gpu_libs/gpu_main/main.cu:103-131).
//
// Hand-off.  For each loop the leader thread writes the command (body,
// argument, iteration count) into every helper block's shared memory through
// distributed shared memory (mapa + st.shared::cluster) and arrives on the
// helper's `cl_go` mbarrier with cluster-scope release; the helper's thread 0
// waits on its own barrier (acquire) and releases its block.  Iteration i of
// the loop runs on thread i mod (C*T) of the cluster.  Each helper block
// reports the end of its share with a release add on the rank's counter in
// global memory (Job::cl_done), which the leader thread polls: a helper never
// accesses the leader block's shared memory, so the leader block may leave
// the kernel whatever its helpers do.  The leader tells the helpers to leave
// (OP_EXIT) before it ends, and writes to a helper block only while that
// block waits for commands, which it does until it receives OP_EXIT.
//
// Every wait is bounded: the leader's by the job timeout and the abort flag;
// a helper's idle wait by the abort flag plus twice the job timeout after it
// (the leader's own waits end within one timeout of an abort).
#include "rt.cuh"

namespace gm {

static __device__ __forceinline__ u32 smem_addr(const void* p) { return (u32)__cvta_generic_to_shared(p); }

// Address of the same shared-memory location in block `cta` of the cluster.
static __device__ __forceinline__ u32 cluster_peer(u32 local, u32 cta) {
    u32 r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(cta));
    return r;
}

__device__ void cluster_setup(int tid) {
    BlockCtx& b = bctx();
    if (b.cl_n <= 1) return;
    if (tid == 0 && b.cl_rank > 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&b.cl_go)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // no block of the cluster writes another's shared memory before every
    // block has initialised its barrier
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// Leader thread: hand command `op` to every helper block.
static __device__ void cluster_post(int op, u64 a0, u64 a1, u64 a2) {
    BlockCtx& b = bctx();
    const u32 cmd = smem_addr(&b.cl_cmd);
    const u32 go = smem_addr(&b.cl_go);
    for (int k = 1; k < b.cl_n; k++) {
        const u32 c = cluster_peer(cmd, (u32)k);
        asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(c + (u32)offsetof(BlockCtx::ClusterCmd, a)), "l"(a0)
                     : "memory");
        asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(c + (u32)offsetof(BlockCtx::ClusterCmd, a) + 8u),
                     "l"(a1)
                     : "memory");
        asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(c + (u32)offsetof(BlockCtx::ClusterCmd, a) + 16u),
                     "l"(a2)
                     : "memory");
        asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(c + (u32)offsetof(BlockCtx::ClusterCmd, op)), "r"(op)
                     : "memory");
        asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_peer(go, (u32)k))
                     : "memory");
    }
}

// Every thread of the leader block: run a parallel loop over the whole cluster.
__device__ int cluster_parfor(void (*body)(long, void*), void* arg, long n, int tid, int T) {
    BlockCtx& b = bctx();
    const int C = b.cl_n;
    if (tid == 0) {
        b.cl_phase++;
        cluster_post(OP_PARFOR, (u64)body, (u64)arg, (u64)n);
    }
    const long stride = (long)T * C;
    for (long i = tid; i < n; i += stride) body(i, arg);
    int rc = MPI_SUCCESS;
    if (tid == 0) {
        Job* j = b.job;
        const u64 want = (u64)b.cl_phase * (u64)(C - 1);
        const u64* cnt = &j->cl_done[b.rank];
        const u64 t0 = gtime();
        for (unsigned it = 0; ld_acquire(cnt) < want; it++) {
            if ((it & 63u) == 63u) {
                if (job_aborted(j)) {
                    rc = GPUMPI_ERR_ABORTED;
                    break;
                }
                if (gtime() - t0 > j->timeout_ns) {
                    job_fail(j, b.rank, GPUMPI_ERR_TIMEOUT, "helper blocks of a cluster rank did not finish a loop");
                    rc = GPUMPI_ERR_TIMEOUT;
                    break;
                }
            }
        }
    }
    return (int)bcast(rc, tid);
}

__device__ void cluster_release() {
    BlockCtx& b = bctx();
    if (b.cl_n <= 1 || b.cl_rank != 0 || b.cl_released) return;
    b.cl_released = 1;
    cluster_post(OP_EXIT, 0, 0, 0);
}

// Thread 0 of a helper block: wait for the next phase of cl_go.  Returns
// false when the wait gave up.
static __device__ bool helper_wait(u32 bar, u32 parity) {
    BlockCtx& b = bctx();
    const Job* j = b.job;
    u64 aborted_at = 0;
    for (unsigned it = 0;; it++) {
        u32 done = 0;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2; "
            "selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u) {
            if (!aborted_at) {
                if (job_aborted(j)) aborted_at = gtime();
            } else if (gtime() - aborted_at > 2 * j->timeout_ns) {
                return false;
            }
        }
    }
}

__device__ void cluster_helper_loop() {
    BlockCtx& b = bctx();
    const int tid = (int)threadIdx.x, T = b.T, C = b.cl_n;
    const u32 go = smem_addr(&b.cl_go);
    __shared__ int s_ok;
    for (u32 parity = 0;; parity ^= 1u) {
        if (tid == 0) s_ok = helper_wait(go, parity);
        __syncthreads();
        if (!s_ok || b.cl_cmd.op != OP_PARFOR) break;
        void (*body)(long, void*) = (void (*)(long, void*))b.cl_cmd.a[0];
        void* arg = (void*)b.cl_cmd.a[1];
        const long n = (long)b.cl_cmd.a[2];
        for (long i = (long)b.cl_rank * T + tid; i < n; i += (long)T * C) body(i, arg);
        __syncthreads();
        if (tid == 0) {
            __threadfence();
            asm volatile("red.release.gpu.global.add.u64 [%0], 1;" ::"l"(&b.job->cl_done[b.rank]) : "memory");
        }
    }
}

}  // namespace gm
