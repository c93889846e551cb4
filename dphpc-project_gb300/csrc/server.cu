// Device side of the serving runtime: the admin block and the worker blocks'
// hand-off (the worker kernel itself is in prog_entry.cu, next to the
// program's __gpu_main).
//
// The reference had a device->host queue in managed memory that the host
// polled (gpu_libs/gpu_libc/cuda_mpi.cuh:392-435, gpu_libs/gpu_main/
// main.cu:294-301) and ran one program per process.  Here one persistent
// launch serves many jobs: the only system-scope traffic is the admin block's
// polling of the admission ring and its completion records; workers wait on
// device memory.  Every job keeps its own memory (mailboxes, tables, heap,
// output) in the HBM pool for its whole life; a worker block runs one rank of
// one job at a time, in the rank slot the admin block gives it, so the
// converted globals of ranks that run at the same time never alias.  Rank
// slots map to worker blocks so that consecutive slots sit on different SMs
// (the host orders the blocks by the SM each reports at start): the ranks of
// one job, which take consecutive slots, spread over the GPU.
#include "rt.cuh"

namespace gm {

static __device__ __forceinline__ u64 ld_acquire_sys(const u64* p) {
    u64 v;
    asm volatile("ld.acquire.sys.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
static __device__ __forceinline__ int ld_volatile_int(const int* p) { return *(const volatile int*)p; }
static __device__ __forceinline__ void st_release_sys(u64* p, u64 v) {
    asm volatile("st.release.sys.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Admin block (every thread).  Thread 0 polls the rings and hands out the
// ranks of admitted jobs (whose memory the host initialised with copies
// before posting them).  Ends when the host asked to stop and nothing runs,
// or on a kill.
__device__ void server_admin(const ServerArgs& A) {
    const int tid = (int)threadIdx.x, T = (int)blockDim.x;
    __shared__ int s_op;   // 0 nothing, 1 admit s_rec, 2 end
    __shared__ AdmitRec s_rec;
    ServeRing* ring = A.ring;
    u64 consumed = 0, posted = 0, seq = 0;
    int nactive = 0;
    unsigned idle_ns = 256;
    for (;;) {
        if (tid == 0) {
            s_op = 0;
            // finished jobs: every rank ran rank_finish (it counts status[3] up last)
            for (int i = 0; i < nactive;) {
                ServeActive& a = A.active[i];
                if (ld_acquire_int(&a.job->status[3]) >= a.nranks) {
                    const u64 k = posted % SERVE_RING;
                    *(volatile u64*)&ring->done[k] = a.ticket;
                    posted++;
                    st_release_sys(&ring->done_head, posted);
                    A.active[i] = A.active[nactive - 1];
                    nactive--;
                    idle_ns = 256;
                } else {
                    i++;
                }
            }
            const u64 head = ld_acquire_sys(&ring->sub_head);
            if (ld_volatile_int(&ring->kill)) {
                s_op = 2;
            } else if (consumed < head && nactive < SERVE_MAX_JOBS) {
                const volatile AdmitRec* r = &ring->sub[consumed % SERVE_RING];
                s_rec.job = r->job;
                s_rec.slot_base = r->slot_base;
                s_rec.nranks = r->nranks;
                s_rec.ticket = r->ticket;
                consumed++;
                s_op = 1;
            } else if (consumed == head && nactive == 0 && ld_volatile_int(&ring->stop)) {
                s_op = 2;
            } else {
                __nanosleep(idle_ns);
                if (idle_ns < 4096) idle_ns <<= 1;
            }
        }
        __syncthreads();
        const int op = s_op;
        if (op == 2) {
            // a kill also ends the running jobs: their waits see the abort flag
            if (tid == 0)
                for (int i = 0; i < nactive; i++) job_fail(A.active[i].job, -1, GPUMPI_ERR_ABORTED, "server killed");
            break;
        }
        if (op == 1) {
            if (tid == 0) {
                __threadfence();
                seq++;
                for (int r = 0; r < s_rec.nranks; r++) {
                    const int sl = s_rec.slot_base + r;
                    const int w = A.perm[sl];
                    A.assign_job[w] = s_rec.job;
                    A.assign_rank[w] = r;
                    A.assign_slot[w] = sl;
                    __threadfence();
                    st_release(&A.assign_seq[w], seq);
                }
                A.active[nactive].job = s_rec.job;
                A.active[nactive].nranks = s_rec.nranks;
                A.active[nactive].slot_base = s_rec.slot_base;
                A.active[nactive].ticket = s_rec.ticket;
                nactive++;
                idle_ns = 256;
            }
        }
        __syncthreads();
    }
    // every worker block leaves once it is idle
    __threadfence();
    for (int w = tid; w < A.nworkers; w += T) st_release(&A.assign_seq[w], ~0ull);
}

// Worker block (every thread): wait for the next rank handed to block w (a
// poll of device memory only).  False once the server ends.
__device__ bool server_take(const ServerArgs& A, int w, u64* seen, Job** job, int* rank, int* slot) {
    __shared__ Job* s_job;
    __shared__ int s_rank, s_slot;
    if (threadIdx.x == 0) {
        unsigned ns = 128;
        u64 v;
        while ((v = ld_acquire(&A.assign_seq[w])) == *seen) {
            __nanosleep(ns);
            if (ns < 2048) ns <<= 1;
        }
        *seen = v;
        s_job = v == ~0ull ? nullptr : A.assign_job[w];
        s_rank = A.assign_rank[w];
        s_slot = A.assign_slot[w];
    }
    __syncthreads();
    *job = s_job;
    *rank = s_rank;
    *slot = s_slot;
    __syncthreads();
    return *job != nullptr;
}

}  // namespace gm
