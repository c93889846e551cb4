// Block-wide execution of one MPI call.  The leader (thread 0) writes the call
// into shared memory and every thread of the rank block runs dispatch_all();
// kernels of the host collective API call the collective functions directly.
#include "rt.cuh"

namespace gm {

static __device__ int finalize_block(int tid, int T) {
    BlockCtx& b = bctx();
    RankPriv* p = b.priv;
    // Deliver every deferred send before leaving (MPI requires completion).
    u64 t0 = gtime();
    for (;;) {
        int pending = (int)bcast(tid == 0 ? (p->defer_head >= 0) : 0, tid);
        if (!pending) break;
        int did = 0;
        p2p_progress(tid, T, &did);
        int code = 0;
        if (tid == 0) {
            if (job_aborted(b.job)) code = GPUMPI_ERR_ABORTED;
            else if (gtime() - t0 > b.job->timeout_ns) {
                job_fail(b.job, b.rank, GPUMPI_ERR_TIMEOUT, "MPI_Finalize: undelivered sends");
                code = GPUMPI_ERR_TIMEOUT;
            } else if (!did) __nanosleep(200);
        }
        code = (int)bcast(code, tid);
        if (code) return code;
    }
    return coll_barrier(&p->comms[0], tid, T);
}

__device__ __noinline__ int dispatch_all(int tid) {
    __syncwarp();
    BlockCtx& b = bctx();
    const int T = b.T;
    Call& c = b.call;
    int rc = MPI_SUCCESS;
    switch (c.op) {
        case OP_SEND_START: rc = p2p_send_start((MPI_Request_impl*)c.a[0], tid, T); break;
        case OP_RECV_POST: rc = p2p_recv_post((MPI_Request_impl*)c.a[0], tid, T); break;
        case OP_WAIT: rc = p2p_wait((MPI_Request_impl*)c.a[0], tid, T, 1); break;
        case OP_TEST: rc = p2p_wait((MPI_Request_impl*)c.a[0], tid, T, 0); break;
        case OP_PROBE:
            rc = p2p_probe((int)c.a[2], (int)c.a[3], (int)c.a[4], (int)c.a[5], (MPI_Status*)c.a[0],
                           tid, T);
            break;
        case OP_BARRIER: rc = coll_barrier((MPI_Comm_impl*)c.a[0], tid, T); break;
        case OP_BCAST: rc = coll_bcast(c.ca, tid, T); break;
        case OP_REDUCE: rc = coll_reduce(c.ca, tid, T); break;
        case OP_ALLREDUCE: rc = coll_allreduce(c.ca, tid, T); break;
        case OP_GATHERV: rc = coll_gatherv(c.ca, tid, T); break;
        case OP_SCATTERV: rc = coll_scatterv(c.ca, tid, T); break;
        case OP_ALLGATHERV: rc = coll_allgatherv(c.ca, tid, T); break;
        case OP_ALLTOALLV: rc = coll_alltoallv(c.ca, tid, T); break;
        case OP_REDUCE_SCATTER_BLOCK: rc = coll_reduce_scatter_block(c.ca, tid, T); break;
        case OP_SCAN: rc = coll_scan(c.ca, (int)c.ca.a0, tid, T); break;
        case OP_COMM_SPLIT: {
            MPI_Comm_impl* out = nullptr;
            rc = comm_split_block((MPI_Comm_impl*)c.a[0], (int)(long long)c.a[1],
                                  (int)(long long)c.a[2], &out, tid, T);
            if (tid == 0) c.a[3] = (u64)out;
            break;
        }
        case OP_MEMCPY: blk_copy((void*)c.a[0], (const void*)c.a[1], c.a[2], tid, T); break;
        case OP_MEMSET: blk_memset((void*)c.a[0], (int)c.a[1], c.a[2], tid, T); break;
        case OP_FINALIZE: rc = finalize_block(tid, T); break;
        case OP_PARFOR: {
            // every thread of the rank block runs a share of the iterations
            void (*body)(long, void*) = (void (*)(long, void*))c.a[0];
            void* arg = (void*)c.a[1];
            const long n = (long)c.a[2];
            if (b.cl_n > 1) rc = cluster_parfor(body, arg, n, tid, T);   // the rank's helper blocks take shares
            else
                for (long i = tid; i < n; i += T) body(i, arg);
            break;
        }
        default: rc = MPI_ERR_INTERN; break;
    }
    bsync();
    if (tid == 0) {
        c.ret = rc;
        // The lists of posted receives and deferred sends change only in these
        // calls; the blocking small-message paths run only while both are empty.
        if (c.op == OP_SEND_START || c.op == OP_RECV_POST || c.op == OP_WAIT || c.op == OP_TEST ||
            c.op == OP_PROBE || c.op == OP_FINALIZE) {
            RankPriv* p = b.priv;
            b.p2p_quiet = p->recv_head < 0 && p->defer_head < 0;
        }
    }
    return rc;
}

}  // namespace gm
