// Host-driven collectives: communicators whose ranks are thread blocks, and
// plans that run a list of collective calls either as one kernel launch per
// call ("plain") or as one persistent cooperative launch in which the blocks
// of every communicator run their communicator's calls in order ("batched").
// Both forms execute the same device schedules as the MPI_* calls of
// converted programs (coll.cu), so their results are identical and their
// speed differs only by launch structure.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <vector>

#include "gpumpi.h"
#include "hostjob.h"
#include "rt.cuh"

extern __device__ MPI_Op_impl gm_builtin_ops[GPUMPI_NUM_BUILTIN_OPS];

namespace gm {

struct DevDesc {
    int op;
    int dtype;
    int redop;
    int root;
    u64 count;
    int comm;       // index into the plan's communicator table
    int esize;
    int algo;
    int sync;       // 1: flag rounds even when the launch is launch-ordered
    void** sbufs;   // [P] device array
    void** rbufs;   // [P]
    const Pub* pub; // [P] buffer table of the launch-ordered forms (nullptr: none)
};

struct DevComm {
    MPI_Comm_impl* handles;   // [P] per-rank handles (sequence numbers persist)
    int size;
    int pad;
};

struct PlanArgs {
    Job* job;
    const DevDesc* descs;
    const int* comm_first;    // [ncomm + 1]: descriptor range of each communicator
    const int* slot_comm;     // [nslots], nullptr = every block in communicator 0
    const int* slot_rank;     // [nslots], nullptr = rank is blockIdx.x
    const DevComm* comms;
    int ordered;              // 1: the launch-ordered forms (calls touch disjoint memory)
    int pad;
};

static __device__ int run_desc(const DevDesc& d, MPI_Comm_impl* comm, int P, int rank, int ordered, int tid,
                               int T) {
    CollArgs a;
    memset(&a, 0, sizeof(a));
    a.comm = comm;
    a.root = d.root;
    a.algo = d.algo;
    a.ssize = a.rsize = d.esize;
    a.dtype = (MPI_Datatype)d.dtype;
    a.op = &gm_builtin_ops[d.redop];
    a.opi = d.redop;
    a.ufn = nullptr;
    const void* sb = d.sbufs ? ldcg(&d.sbufs[rank]) : nullptr;
    void* rb = d.rbufs ? ldcg(&d.rbufs[rank]) : nullptr;
    if (ordered && d.pub && !d.sync) {
        a.sbuf = sb;
        a.rbuf = rb;
        switch (d.op) {
            case GPUMPI_COLL_BCAST:
                if (d.algo == 2) break;   // the tree forwards copies made in this launch: flag rounds
                a.count = d.count * d.esize;
                return coll_lo_bcast(a, d.pub, P, rank, tid, T);
            case GPUMPI_COLL_REDUCE:
                a.count = d.count;
                return coll_lo_reduce(a, d.pub, P, rank, tid, T);
            case GPUMPI_COLL_ALLREDUCE:
                a.count = d.count;
                return coll_lo_allreduce(a, d.pub, P, rank, tid, T);
            case GPUMPI_COLL_ALLTOALL:
            case GPUMPI_COLL_ALLGATHER:
                a.count = d.count;
                return coll_lo_alltoall(a, d.pub, P, rank, d.op == GPUMPI_COLL_ALLGATHER, tid, T);
            default: break;   // a barrier keeps its flag round
        }
    }
    switch (d.op) {
        case GPUMPI_COLL_BARRIER: return coll_barrier(comm, tid, T);
        case GPUMPI_COLL_BCAST:
            a.rbuf = rb;
            a.count = d.count * d.esize;
            return coll_bcast(a, tid, T);
        case GPUMPI_COLL_REDUCE:
            a.sbuf = sb;
            a.rbuf = rb;
            a.count = d.count;
            return coll_reduce(a, tid, T);
        case GPUMPI_COLL_ALLREDUCE:
            a.sbuf = sb;
            a.rbuf = rb;
            a.count = d.count;
            return coll_allreduce(a, tid, T);
        case GPUMPI_COLL_ALLTOALL:
            a.sbuf = sb;
            a.rbuf = rb;
            a.a0 = (long long)d.count;
            a.a1 = (long long)d.count;
            return coll_alltoallv(a, tid, T);
        case GPUMPI_COLL_ALLGATHER:
            a.sbuf = sb;
            a.rbuf = rb;
            a.a0 = (long long)d.count;
            a.a1 = (long long)d.count;
            return coll_allgatherv(a, tid, T);
        default: return MPI_ERR_ARG;
    }
}

extern "C" __global__ void __launch_bounds__(1024) gpumpi_plan_kernel(PlanArgs A) {
    BlockCtx& b = bctx();
    const int slot = blockIdx.x;
    const int c = A.slot_comm ? A.slot_comm[slot] : 0;
    const int rank = A.slot_rank ? A.slot_rank[slot] : slot;
    if (threadIdx.x == 0) {
        b.job = A.job;
        b.priv = nullptr;
        b.rank = rank;
        b.slot = slot;
        b.T = (int)blockDim.x;
        b.leader_mode = 0;
        b.in_call = 0;
        b.bulk_broken = 0;
        b.lazy_n = 0;
        b.sc_handle = nullptr;
        b.mb_cluster = 0;
        b.mb_local = nullptr;
        b.cl_n = 1;
        b.cl_rank = 0;
    }
    __syncthreads();
    MPI_Comm_impl* comm = &A.comms[c].handles[rank];
    const int tid = (int)threadIdx.x, T = (int)blockDim.x;
    const int P = A.comms[c].size;
    for (int i = A.comm_first[c]; i < A.comm_first[c + 1]; i++) {
        if (run_desc(A.descs[i], comm, P, rank, A.ordered, tid, T) != MPI_SUCCESS) break;
    }
}

}  // namespace gm

using namespace gm;

// ------------------------------------------------------------------ host side
struct gpumpi_comm_s {
    int n;
    char* base;          // device allocation
    DevComm* dcomm;      // device DevComm
    DevComm hcomm;
};

struct gpumpi_plan_s {
    int ndesc;
    int ncomm;
    int batched;
    int threads;
    size_t smem;
    char* base;                       // device allocation
    PlanArgs batch_args;              // batched launch
    std::vector<PlanArgs> plain_args; // one per descriptor
    std::vector<int> plain_grid;
    std::vector<int> plain_threads;   // threads per rank of each plain launch
    std::vector<size_t> plain_smem;   // dynamic shared memory of each plain launch
    int total_slots;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<gpumpi_coll_desc> descs;   // host copies for the host-buffer path
    std::vector<std::vector<void*>> sb, rb;
    int independent = 0;                   // calls touch disjoint memory and include no barrier
    int sync_mode = 0;                     // 0 automatic, 1 flag rounds for every call
    std::vector<int> plain_op;             // collective of each plain launch
};

namespace {

std::atomic<unsigned long long> g_launches{0};

struct ApiJob {
    Job* djob = nullptr;
    int* status = nullptr;
    char* err = nullptr;
};
ApiJob g_api;

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[300];                                                                 \
            snprintf(m_, sizeof(m_), "%s: %s", #call, cudaGetErrorString(e_));            \
            set_last_error(m_);                                                           \
            return GPUMPI_ECUDA;                                                          \
        }                                                                                 \
    } while (0)

int api_job() {
    if (g_api.djob) return GPUMPI_OK;
    // the plan kernel streams through L2 (ld.global.cg) and stages bulk copies
    // in shared memory: prefer the largest shared-memory carve-out
    CK(cudaFuncSetAttribute((const void*)gpumpi_plan_kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                            (int)cudaSharedmemCarveoutMaxShared));
    Job hj;
    memset(&hj, 0, sizeof(hj));
    char* mem = nullptr;
    CK(cudaMalloc(&mem, sizeof(Job) + 64 + 256));
    CK(cudaMemset(mem, 0, sizeof(Job) + 64 + 256));
    hj.id = -1;
    hj.timeout_ns = 30ull * 1000000000ull;
    hj.status = (int*)(mem + sizeof(Job));
    hj.err_msg = mem + sizeof(Job) + 64;
    CK(cudaMemcpy(mem, &hj, sizeof(Job), cudaMemcpyHostToDevice));
    g_api.djob = (Job*)mem;
    g_api.status = hj.status;
    g_api.err = hj.err_msg;
    return GPUMPI_OK;
}

int esize_of(int dtype) {
    switch (dtype) {
        case MPI_CHAR: case MPI_SIGNED_CHAR: case MPI_UNSIGNED_CHAR: case MPI_BYTE: case MPI_INT8_T:
        case MPI_UINT8_T: case MPI_C_BOOL: return 1;
        case MPI_SHORT: case MPI_UNSIGNED_SHORT: case MPI_INT16_T: case MPI_UINT16_T: return 2;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: case MPI_INT32_T: case MPI_UINT32_T: return 4;
        case MPI_LONG: case MPI_LONG_LONG_INT: case MPI_LONG_LONG: case MPI_UNSIGNED_LONG:
        case MPI_UNSIGNED_LONG_LONG: case MPI_DOUBLE: case MPI_INT64_T: case MPI_UINT64_T: return 8;
        default: return -1;
    }
}

// Bytes a rank sends / receives for a descriptor.
void desc_bytes(const gpumpi_coll_desc& d, int P, size_t* in, size_t* out) {
    size_t e = (size_t)esize_of(d.dtype) * d.count;
    switch (d.op) {
        case GPUMPI_COLL_BCAST: *in = e; *out = e; break;
        case GPUMPI_COLL_REDUCE:
        case GPUMPI_COLL_ALLREDUCE: *in = e; *out = e; break;
        case GPUMPI_COLL_ALLTOALL: *in = e * P; *out = e * P; break;
        case GPUMPI_COLL_ALLGATHER: *in = e; *out = e * P; break;
        default: *in = *out = 0;
    }
}

// True when no call of the list writes memory that another call reads or
// writes (and none is a barrier): the plan kernel may then run every call in
// its launch-ordered form.  Each call's spans: the bytes each rank reads and
// writes (Bcast: the root's buffer is read, the others written).  Spans of one
// call never conflict with each other here (in-place forms are the
// schedules' concern); spans are sorted by start and compared with the spans
// still open.
bool plan_independent(const gpumpi_coll_desc* descs, int ndesc) {
    struct Span {
        uintptr_t lo, hi;
        int call, w;
    };
    std::vector<Span> v;
    for (int i = 0; i < ndesc; i++) {
        const gpumpi_coll_desc& d = descs[i];
        if (d.op == GPUMPI_COLL_BARRIER) return false;
        const int P = d.comm->n;
        const size_t e = (size_t)esize_of(d.dtype) * d.count;
        auto add = [&](void* const* tab, int r, size_t bytes, int w) {
            const void* p = tab ? tab[r] : nullptr;
            if (p && bytes) v.push_back({(uintptr_t)p, (uintptr_t)p + bytes, i, w});
        };
        for (int r = 0; r < P; r++) {
            switch (d.op) {
                case GPUMPI_COLL_BCAST: add(d.recvbufs, r, e, r != d.root); break;
                case GPUMPI_COLL_REDUCE:
                    add(d.sendbufs, r, e, 0);
                    if (r == d.root) add(d.recvbufs, r, e, 1);
                    break;
                case GPUMPI_COLL_ALLREDUCE:
                    add(d.sendbufs, r, e, 0);
                    add(d.recvbufs, r, e, 1);
                    break;
                case GPUMPI_COLL_ALLTOALL:
                    add(d.sendbufs, r, e * P, 0);
                    add(d.recvbufs, r, e * P, 1);
                    break;
                case GPUMPI_COLL_ALLGATHER:
                    add(d.sendbufs, r, e, 0);
                    add(d.recvbufs, r, e * P, 1);
                    break;
                default: break;
            }
        }
    }
    std::sort(v.begin(), v.end(), [](const Span& a, const Span& b) { return a.lo < b.lo; });
    std::vector<Span> open;
    for (const Span& x : v) {
        size_t k = 0;
        for (size_t j = 0; j < open.size(); j++)
            if (open[j].hi > x.lo) open[k++] = open[j];
        open.resize(k);
        for (const Span& o : open)
            if (o.call != x.call && (o.w || x.w)) return false;
        open.push_back(x);
    }
    return true;
}

int launch(const void* kern, int grid, int threads, size_t smem, PlanArgs* args, cudaStream_t st) {
    void* params[] = {args};
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    CK(cudaLaunchKernelExC(&cfg, kern, params));
    g_launches++;
    return GPUMPI_OK;
}

}  // namespace

extern "C" int gpumpi_comm_create(int nranks, gpumpi_comm_t* out) {
    if (nranks <= 0 || !out) return GPUMPI_EINVAL;
    int rc = api_job();
    if (rc) return rc;
    const size_t n = (size_t)nranks;
    size_t off_cs = 0;
    size_t off_pub = 256;
    size_t off_flags = off_pub + ((sizeof(Pub) * n + 255) & ~(size_t)255);
    size_t off_h = off_flags + ((3 * sizeof(u64) * n + 255) & ~(size_t)255);
    size_t off_dc = off_h + ((sizeof(MPI_Comm_impl) * n + 255) & ~(size_t)255);
    size_t total = off_dc + 256;
    char* base = nullptr;
    CK(cudaMalloc(&base, total));
    CK(cudaMemset(base, 0, total));
    CommShared cs;
    memset(&cs, 0, sizeof(cs));
    cs.size = nranks;
    cs.ctx = 1;
    cs.members = nullptr;
    cs.pub = (Pub*)(base + off_pub);
    cs.arrive = (u64*)(base + off_flags);
    cs.mid = cs.arrive + n;
    cs.depart = cs.arrive + 2 * n;
    CK(cudaMemcpy(base + off_cs, &cs, sizeof(cs), cudaMemcpyHostToDevice));
    std::vector<MPI_Comm_impl> h(n);
    for (int r = 0; r < nranks; r++) {
        h[r].kind = 1;
        h[r].ctx = 1;
        h[r].size = nranks;
        h[r].rank = r;
        h[r].refcnt = 1;
        h[r].pad = 0;
        h[r].cs = (CommShared*)(base + off_cs);
        h[r].seq = 0;
    }
    CK(cudaMemcpy(base + off_h, h.data(), sizeof(MPI_Comm_impl) * n, cudaMemcpyHostToDevice));
    gpumpi_comm_s* c = new gpumpi_comm_s();
    c->n = nranks;
    c->base = base;
    c->hcomm.handles = (MPI_Comm_impl*)(base + off_h);
    c->hcomm.size = nranks;
    c->hcomm.pad = 0;
    c->dcomm = (DevComm*)(base + off_dc);
    CK(cudaMemcpy(c->dcomm, &c->hcomm, sizeof(DevComm), cudaMemcpyHostToDevice));
    *out = c;
    return GPUMPI_OK;
}

extern "C" int gpumpi_comm_destroy(gpumpi_comm_t c) {
    if (!c) return GPUMPI_EINVAL;
    cudaFree(c->base);
    delete c;
    return GPUMPI_OK;
}

extern "C" int gpumpi_comm_size(gpumpi_comm_t c, int* n) {
    if (!c || !n) return GPUMPI_EINVAL;
    *n = c->n;
    return GPUMPI_OK;
}

extern "C" int gpumpi_plan_create(const gpumpi_coll_desc* descs, int ndesc, int threads, int batched,
                                  gpumpi_plan_t* out) {
    return gpumpi_plan_create_ex(descs, ndesc, threads, batched, nullptr, out);
}

extern "C" int gpumpi_plan_create_ex(const gpumpi_coll_desc* descs, int ndesc, int threads, int batched,
                                     const int* plain_threads, gpumpi_plan_t* out) {
    if (!descs || ndesc <= 0 || !out) return GPUMPI_EINVAL;
    if (threads == 0) threads = 128;
    if (threads < 64 || threads > 1024 || threads % 32) return GPUMPI_EINVAL;
    for (int i = 0; plain_threads && i < ndesc; i++) {
        const int t = plain_threads[i];
        if (t != 0 && (t < 64 || t > 1024 || t % 32)) return GPUMPI_EINVAL;
    }
    int rc = api_job();
    if (rc) return rc;
    // communicators in order of first use; descriptors grouped by communicator, order kept
    std::vector<gpumpi_comm_t> comms;
    std::vector<int> cidx(ndesc);
    for (int i = 0; i < ndesc; i++) {
        const gpumpi_coll_desc& d = descs[i];
        if (!d.comm || esize_of(d.dtype) < 0 || d.op < 0 || d.op > GPUMPI_COLL_ALLGATHER) return GPUMPI_EINVAL;
        if ((d.op == GPUMPI_COLL_REDUCE || d.op == GPUMPI_COLL_ALLREDUCE) && (d.redop < 0 || d.redop > 3))
            return GPUMPI_EINVAL;
        if ((d.op == GPUMPI_COLL_BCAST || d.op == GPUMPI_COLL_REDUCE) && (d.root < 0 || d.root >= d.comm->n))
            return GPUMPI_EINVAL;
        if (d.algo < 0 || d.algo > 4) return GPUMPI_EINVAL;
        auto it = std::find(comms.begin(), comms.end(), d.comm);
        cidx[i] = (int)(it - comms.begin());
        if (it == comms.end()) comms.push_back(d.comm);
    }
    const int ncomm = (int)comms.size();
    std::vector<int> order(ndesc);
    for (int i = 0; i < ndesc; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cidx[a] < cidx[b]; });
    std::vector<int> comm_first(ncomm + 1, 0);
    for (int i = 0; i < ndesc; i++) comm_first[cidx[i] + 1]++;
    for (int c = 0; c < ncomm; c++) comm_first[c + 1] += comm_first[c];
    int total_slots = 0;
    for (auto* c : comms) total_slots += c->n;
    size_t ptrs = 0;
    for (int i = 0; i < ndesc; i++) ptrs += 2 * (size_t)descs[i].comm->n;
    // device layout: descs | comm_first | slot_comm | slot_rank | comms | per-desc comm_first pairs | pointers
    size_t off_desc = 0;
    size_t off_cf = off_desc + sizeof(DevDesc) * ndesc;
    size_t off_sc = (off_cf + sizeof(int) * (ncomm + 1) + 15) & ~(size_t)15;
    size_t off_sr = off_sc + sizeof(int) * total_slots;
    size_t off_cm = (off_sr + sizeof(int) * total_slots + 15) & ~(size_t)15;
    size_t off_pp = off_cm + sizeof(DevComm) * ncomm;
    size_t off_pc = (off_pp + sizeof(int) * 2 * ndesc + 15) & ~(size_t)15;
    size_t off_ptr = off_pc + sizeof(DevComm) * ndesc;
    size_t off_pubt = (off_ptr + sizeof(void*) * ptrs + 63) & ~(size_t)63;   // Pub tables, one entry per rank
    size_t total = off_pubt + sizeof(Pub) * (ptrs / 2) + 16;
    gpumpi_plan_s* p = new gpumpi_plan_s();
    CK(cudaMalloc(&p->base, total));
    char* base = p->base;
    std::vector<char> h(total, 0);
    DevDesc* hd = (DevDesc*)(h.data() + off_desc);
    void** hp = (void**)(h.data() + off_ptr);
    Pub* hpub = (Pub*)(h.data() + off_pubt);
    size_t pk = 0, pubk = 0;
    p->descs.assign(descs, descs + ndesc);
    p->sb.resize(ndesc);
    p->rb.resize(ndesc);
    for (int k = 0; k < ndesc; k++) {
        const int i = order[k];
        const gpumpi_coll_desc& d = descs[i];
        const int P = d.comm->n;
        DevDesc& x = hd[k];
        x.op = d.op;
        x.dtype = d.dtype;
        x.redop = d.redop;
        x.root = d.root;
        x.count = d.count;
        x.comm = cidx[i];
        x.esize = esize_of(d.dtype);
        x.algo = d.algo;
        x.sync = d.sync ? 1 : 0;
        x.sbufs = (void**)(base + off_ptr + sizeof(void*) * pk);
        for (int r = 0; r < P; r++) hp[pk++] = d.sendbufs ? d.sendbufs[r] : nullptr;
        x.rbufs = (void**)(base + off_ptr + sizeof(void*) * pk);
        for (int r = 0; r < P; r++) hp[pk++] = d.recvbufs ? d.recvbufs[r] : nullptr;
        p->sb[i].assign(hp + pk - 2 * P, hp + pk - P);
        p->rb[i].assign(hp + pk - P, hp + pk);
        x.pub = (const Pub*)(base + off_pubt) + pubk;
        for (int r = 0; r < P; r++, pubk++) {
            Pub& e = hpub[pubk];
            e.rbuf = d.recvbufs ? d.recvbufs[r] : nullptr;
            e.sbuf = d.sendbufs ? d.sendbufs[r] : e.rbuf;
            e.a0 = (long long)d.count;
            e.a1 = x.esize;
        }
    }
    memcpy(h.data() + off_cf, comm_first.data(), sizeof(int) * (ncomm + 1));
    int* sc = (int*)(h.data() + off_sc);
    int* sr = (int*)(h.data() + off_sr);
    int s = 0;
    for (int c = 0; c < ncomm; c++)
        for (int r = 0; r < comms[c]->n; r++) {
            sc[s] = c;
            sr[s] = r;
            s++;
        }
    DevComm* hc = (DevComm*)(h.data() + off_cm);
    for (int c = 0; c < ncomm; c++) hc[c] = comms[c]->hcomm;
    // plain launches: each descriptor alone, its own communicator at index 0
    int* pp = (int*)(h.data() + off_pp);
    DevComm* pc = (DevComm*)(h.data() + off_pc);
    for (int k = 0; k < ndesc; k++) {
        pp[2 * k] = 0;
        pp[2 * k + 1] = 1;
        pc[k] = comms[hd[k].comm]->hcomm;
    }
    CK(cudaMemcpy(base, h.data(), total, cudaMemcpyHostToDevice));
    p->ndesc = ndesc;
    p->ncomm = ncomm;
    p->batched = batched;
    p->threads = threads;
    p->smem = rank_smem_bytes(0);
    p->total_slots = total_slots;
    p->batch_args.job = g_api.djob;
    p->batch_args.descs = (const DevDesc*)(base + off_desc);
    p->batch_args.comm_first = (const int*)(base + off_cf);
    p->batch_args.slot_comm = (const int*)(base + off_sc);
    p->batch_args.slot_rank = (const int*)(base + off_sr);
    p->batch_args.comms = (const DevComm*)(base + off_cm);
    p->independent = plan_independent(descs, ndesc) ? 1 : 0;
    p->batch_args.ordered = p->independent;
    p->batch_args.pad = 0;
    p->plain_args.resize(ndesc);
    p->plain_grid.resize(ndesc);
    p->plain_threads.resize(ndesc);
    for (int k = 0; k < ndesc; k++) {
        const int t = plain_threads ? plain_threads[order[k]] : 0;
        p->plain_threads[k] = t ? t : threads;
        PlanArgs& a = p->plain_args[k];
        a.job = g_api.djob;
        a.descs = (const DevDesc*)(base + off_desc) + k;
        a.comm_first = (const int*)(base + off_pp) + 2 * k;
        a.slot_comm = nullptr;
        a.slot_rank = nullptr;
        a.comms = (const DevComm*)(base + off_pc) + k;
        a.ordered = hd[k].op != GPUMPI_COLL_BARRIER;   // one call per launch: always launch-ordered
        a.pad = 0;
        p->plain_op.push_back(hd[k].op);
        p->plain_grid[k] = comms[hd[k].comm]->n;
    }
    // co-residency: every rank block of one launch must fit on the GPU at once
    int per = 0, sms = 0, dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    p->plain_smem.assign(ndesc, rank_smem_bytes(0));
    for (int k = 0; k <= ndesc; k++) {
        // k < ndesc: each plain launch at its own thread count; k == ndesc: the batched launch
        if (k < ndesc && batched) continue;
        if (k == ndesc && !batched) break;
        const int t = k < ndesc ? p->plain_threads[k] : threads;
        const int need = k < ndesc ? p->plain_grid[k] : total_slots;
        const size_t smem = pick_rank_smem((const void*)gpumpi_plan_kernel, t, need);
        if (k < ndesc) p->plain_smem[k] = smem;
        else p->smem = smem;
        CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)gpumpi_plan_kernel, t, smem));
        if ((long long)per * sms < need) {
            char m[200];
            snprintf(m, sizeof(m), "%d rank blocks of %d threads cannot be co-resident (max %d)", need, t,
                     per * sms);
            set_last_error(m);
            cudaFree(p->base);
            delete p;
            return GPUMPI_ENORES;
        }
    }
    *out = p;
    return GPUMPI_OK;
}

static int plan_enqueue(gpumpi_plan_t p, cudaStream_t st) {
    const void* k = (const void*)gpumpi_plan_kernel;
    if (p->batched) return launch(k, p->total_slots, p->threads, p->smem, &p->batch_args, st);
    for (int i = 0; i < p->ndesc; i++) {
        int rc = launch(k, p->plain_grid[i], p->plain_threads[i], p->plain_smem[i], &p->plain_args[i], st);
        if (rc) return rc;
    }
    return GPUMPI_OK;
}

extern "C" int gpumpi_plan_launch(gpumpi_plan_t p, void* stream) {
    if (!p) return GPUMPI_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    if (p->exec) {
        CK(cudaGraphLaunch(p->exec, st));
        g_launches += p->batched ? 1 : p->ndesc;
        return GPUMPI_OK;
    }
    return plan_enqueue(p, st);
}

extern "C" int gpumpi_plan_set_sync(gpumpi_plan_t p, int mode) {
    if (!p || mode < 0 || mode > 1) return GPUMPI_EINVAL;
    p->sync_mode = mode;
    p->batch_args.ordered = mode == 0 && p->independent;
    for (int k = 0; k < p->ndesc; k++)
        p->plain_args[k].ordered = mode == 0 && p->plain_op[k] != GPUMPI_COLL_BARRIER;
    // a captured graph holds the old launch arguments: launch eagerly until captured again
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    p->exec = nullptr;
    p->graph = nullptr;
    return GPUMPI_OK;
}

extern "C" int gpumpi_plan_launch_ordered(gpumpi_plan_t p) {
    if (!p) return 0;
    return p->batched ? p->batch_args.ordered : (p->sync_mode == 0);
}

extern "C" int gpumpi_plan_capture(gpumpi_plan_t p, void* stream) {
    if (!p) return GPUMPI_EINVAL;
    (void)stream;   // captured on a private stream; replays go to the stream given to gpumpi_plan_launch
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    unsigned long long before = g_launches;
    int rc = plan_enqueue(p, cap);
    g_launches = before;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    CK(e);
    CK(cudaGraphInstantiate(&p->exec, g, 0));
    p->graph = g;
    return GPUMPI_OK;
}

// Host-buffer path: copy every rank's send data from host memory, run the
// plan, copy every rank's result back.  host_send/host_recv hold, for each
// descriptor in the order given to gpumpi_plan_create, one host pointer per
// rank (nullptr = skip).
namespace {

// Copies of one direction, merged while both sides continue where the
// previous copy ended, within one descriptor, the device side inside one
// allocation (cuMemGetAddressRange, fetched through the runtime) and the host
// side of one memory type; rank buffers carved from one allocation on each
// side become one cudaMemcpyAsync.
typedef int (*AddrRangeFn)(unsigned long long* base, size_t* size, unsigned long long ptr);

AddrRangeFn addr_range() {
    static AddrRangeFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (AddrRangeFn)f;
        else
            cudaGetLastError();
    }
    return fn;
}

int host_kind(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return (int)a.type;
}

struct CopyRun {
    char* dst = nullptr;
    const char* src = nullptr;
    size_t n = 0;
    int desc = -1;
    unsigned long long dev_end = 0;   // end of the device allocation of the run
    int hkind = -1;
    int add(int d_idx, void* d, const void* s, size_t len, cudaMemcpyKind kind, cudaStream_t st) {
        const bool to_dev = kind == cudaMemcpyHostToDevice;
        const unsigned long long dptr = (unsigned long long)(to_dev ? (uintptr_t)d : (uintptr_t)s);
        const void* hptr = to_dev ? s : (const void*)d;
        if (n && d_idx == desc && (char*)d == dst + n && (const char*)s == src + n && dptr + len <= dev_end &&
            hkind >= 0 && host_kind(hptr) == hkind) {
            n += len;
            return GPUMPI_OK;
        }
        int rc = flush(kind, st);
        dst = (char*)d;
        src = (const char*)s;
        n = len;
        desc = d_idx;
        dev_end = 0;
        hkind = -1;
        unsigned long long base = 0;
        size_t size = 0;
        AddrRangeFn f = addr_range();
        if (f && f(&base, &size, dptr) == 0) {
            dev_end = base + size;
            hkind = host_kind(hptr);
        }
        return rc;
    }
    int flush(cudaMemcpyKind kind, cudaStream_t st) {
        if (n) CK(cudaMemcpyAsync(dst, src, n, kind, st));
        n = 0;
        return GPUMPI_OK;
    }
};

}  // namespace

extern "C" int gpumpi_plan_run_host(gpumpi_plan_t p, void* const* host_send, void* const* host_recv,
                                    void* stream, uint64_t* h2d_bytes, uint64_t* d2h_bytes) {
    if (!p) return GPUMPI_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    size_t k = 0, bi = 0, bo = 0;
    CopyRun run;
    int rc = GPUMPI_OK;
    for (int d = 0; d < p->ndesc && !rc; d++) {
        const int P = p->descs[d].comm->n;
        size_t in, out;
        desc_bytes(p->descs[d], P, &in, &out);
        for (int r = 0; r < P && !rc; r++, k++) {
            const bool is_bcast = p->descs[d].op == GPUMPI_COLL_BCAST;
            void* dst = is_bcast ? p->rb[d][r] : p->sb[d][r];
            if (is_bcast && r != p->descs[d].root) continue;
            if (host_send && host_send[k] && dst && in) {
                rc = run.add(d, dst, host_send[k], in, cudaMemcpyHostToDevice, st);
                bi += in;
            }
        }
    }
    if (!rc) rc = run.flush(cudaMemcpyHostToDevice, st);
    if (!rc) rc = gpumpi_plan_launch(p, stream);
    if (rc) return rc;
    k = 0;
    for (int d = 0; d < p->ndesc && !rc; d++) {
        const int P = p->descs[d].comm->n;
        size_t in, out;
        desc_bytes(p->descs[d], P, &in, &out);
        for (int r = 0; r < P && !rc; r++, k++) {
            if (p->descs[d].op == GPUMPI_COLL_REDUCE && r != p->descs[d].root) continue;
            if (host_recv && host_recv[k] && p->rb[d][r] && out) {
                rc = run.add(d, host_recv[k], p->rb[d][r], out, cudaMemcpyDeviceToHost, st);
                bo += out;
            }
        }
    }
    if (!rc) rc = run.flush(cudaMemcpyDeviceToHost, st);
    if (rc) return rc;
    if (h2d_bytes) *h2d_bytes = bi;
    if (d2h_bytes) *d2h_bytes = bo;
    return GPUMPI_OK;
}

extern "C" int gpumpi_plan_destroy(gpumpi_plan_t p) {
    if (!p) return GPUMPI_EINVAL;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    cudaFree(p->base);
    delete p;
    return GPUMPI_OK;
}

extern "C" int gpumpi_api_status(char* msg, int len);
static int one_shot(const gpumpi_coll_desc* descs, int ndesc, int threads, void* stream, int batched) {
    gpumpi_plan_t p = nullptr;
    int rc = gpumpi_plan_create(descs, ndesc, threads, batched, &p);
    if (rc) return rc;
    rc = gpumpi_plan_launch(p, stream);
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    gpumpi_plan_destroy(p);
    if (rc) return rc;
    if (e != cudaSuccess) return GPUMPI_ECUDA;
    return gpumpi_api_status(nullptr, 0);
}

extern "C" int gpumpi_coll_plain(const gpumpi_coll_desc* descs, int ndesc, int threads, void* stream) {
    return one_shot(descs, ndesc, threads, stream, 0);
}

extern "C" int gpumpi_coll_batched(const gpumpi_coll_desc* descs, int ndesc, int threads, void* stream) {
    return one_shot(descs, ndesc, threads, stream, 1);
}

// Error state of the collective API's device job; clears it.
extern "C" int gpumpi_api_status(char* msg, int len) {
    if (!g_api.djob) return GPUMPI_OK;
    int st[16];
    CK(cudaMemcpy(st, g_api.status, sizeof(st), cudaMemcpyDeviceToHost));
    if (st[1] == 0) return GPUMPI_OK;
    char m[256];
    CK(cudaMemcpy(m, g_api.err, sizeof(m), cudaMemcpyDeviceToHost));
    m[255] = 0;
    if (msg && len > 0) snprintf(msg, len, "error %d on rank %d: %s", st[1], st[2], m);
    char full[320];
    snprintf(full, sizeof(full), "collective job error %d on rank %d: %s", st[1], st[2], m);
    set_last_error(full);
    CK(cudaMemset(g_api.status, 0, sizeof(st)));
    return GPUMPI_EJOB;
}

extern "C" uint64_t gpumpi_kernel_launches(void) { return g_launches; }

// ------------------------------------------------------------------ allocation-free allreduce
// Some callers may not allocate device memory on their call path: a serving
// loop that reserved all of HBM when it started, a host thread running under
// a pooled allocator's fixed budget, or code that must not block the device
// (cudaMalloc and cudaFree can synchronise it).  gpumpi_allreduce_noalloc
// serves them: it runs the same allreduce schedule as the plan kernel, but
// its synchronisation state (communicator tables, flags, per-rank handles,
// error words) lives in the fixed array below instead of cudaMalloc'd memory.
//
// The array is a file-scope device variable, so every GPU that loads this
// library holds it until the process exits, and every call shares it: each
// call rewrites the part it uses (clearing the flags), and calls whose
// kernels overlap on the GPU race on it.  Host code may not use the array's
// name as a device address; the entry point looks the address up with
// cudaGetSymbolAddress the first time it runs on a device (with that device
// current), so that first call should come before any stream capture.
namespace {

constexpr int NOALLOC_MAX_RANKS = 256;
constexpr size_t NOALLOC_SCRATCH_BYTES = 64 * 1024;

static __device__ __align__(256) unsigned char gm_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

struct NoallocLayout {
    size_t job, status, err, cs, pub, flags, handles, dcomm, desc, first, ptrs, total;
};

constexpr size_t noalloc_take(size_t& o, size_t bytes) {
    o = (o + 255) & ~(size_t)255;
    const size_t at = o;
    o += bytes;
    return at;
}

constexpr NoallocLayout noalloc_layout(int n) {
    NoallocLayout L{};
    size_t o = 0;
    L.job = noalloc_take(o, sizeof(Job));
    L.status = noalloc_take(o, sizeof(int) * 16);
    L.err = noalloc_take(o, 256);
    L.cs = noalloc_take(o, sizeof(CommShared));
    L.pub = noalloc_take(o, sizeof(Pub) * (size_t)n);
    L.flags = noalloc_take(o, sizeof(u64) * 3 * (size_t)n);
    L.handles = noalloc_take(o, sizeof(MPI_Comm_impl) * (size_t)n);
    L.dcomm = noalloc_take(o, sizeof(DevComm));
    L.desc = noalloc_take(o, sizeof(DevDesc));
    L.first = noalloc_take(o, sizeof(int) * 2);
    L.ptrs = noalloc_take(o, sizeof(void*) * 2 * (size_t)n);
    L.total = noalloc_take(o, 0);
    return L;
}

// The layout grows with the rank count; the largest one must fit the array
// (a larger Job, Pub or communicator record fails the build here instead of
// overflowing the array at run time).
static_assert(noalloc_layout(NOALLOC_MAX_RANKS).total <= NOALLOC_SCRATCH_BYTES,
              "allocation-free allreduce: scratch array too small for NOALLOC_MAX_RANKS");

std::mutex g_noalloc_mu;
void* g_noalloc_dev_ptr[64];                                    // per device, looked up once
unsigned char g_noalloc_image[NOALLOC_SCRATCH_BYTES];           // host image of the used prefix

}  // namespace

// See include/gpumpi.h.  Synchronises `stream`; returns 0 or an error code.
extern "C" int gpumpi_allreduce_noalloc(void* const* sendbufs, void* const* recvbufs, int nranks,
                                        uint64_t count, int dtype, int redop, int threads_per_rank,
                                        void* stream) {
    if (nranks < 1 || nranks > NOALLOC_MAX_RANKS) {
        char m[160];
        snprintf(m, sizeof(m), "gpumpi_allreduce_noalloc: %d ranks requested, the fixed scratch holds at most %d",
                 nranks, NOALLOC_MAX_RANKS);
        set_last_error(m);
        return GPUMPI_EINVAL;
    }
    const int es = esize_of(dtype);
    if (!sendbufs || !recvbufs || es < 0 || redop < 0 || redop > 3) {
        set_last_error("gpumpi_allreduce_noalloc: bad buffers, datatype or operator");
        return GPUMPI_EINVAL;
    }
    if (threads_per_rank == 0) threads_per_rank = 128;
    if (threads_per_rank < 64 || threads_per_rank > 1024 || threads_per_rank % 32) {
        set_last_error("gpumpi_allreduce_noalloc: threads_per_rank must be a multiple of 32 in [64, 1024]");
        return GPUMPI_EINVAL;
    }
    for (int r = 0; r < nranks; r++)
        if (!sendbufs[r] || !recvbufs[r]) {
            set_last_error("gpumpi_allreduce_noalloc: a send or receive buffer is NULL");
            return GPUMPI_EINVAL;
        }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_last_error("gpumpi_allreduce_noalloc: device ordinal above 63");
        return GPUMPI_EINVAL;
    }
    if (!g_noalloc_dev_ptr[dev]) {
        void* p = nullptr;
        CK(cudaGetSymbolAddress(&p, gm_noalloc_scratch));
        g_noalloc_dev_ptr[dev] = p;
    }
    char* base = (char*)g_noalloc_dev_ptr[dev];
    const NoallocLayout L = noalloc_layout(nranks);
    if (L.total > NOALLOC_SCRATCH_BYTES) {   // unreachable while the static_assert holds
        set_last_error("gpumpi_allreduce_noalloc: layout exceeds the scratch array");
        return GPUMPI_EINVAL;
    }
    const size_t smem = sizeof(BlockCtx) + 64;
    int per = 0, sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)gpumpi_plan_kernel, threads_per_rank, smem));
    if ((long long)per * sms < nranks) {
        set_last_error("gpumpi_allreduce_noalloc: rank blocks cannot all be resident");
        return GPUMPI_ENORES;
    }
    // Build the used prefix on the host (zeros clear the flags), then copy it.
    unsigned char* img = g_noalloc_image;
    memset(img, 0, L.total);
    Job& job = *(Job*)(img + L.job);
    job.id = -2;
    job.timeout_ns = 30ull * 1000000000ull;
    job.status = (int*)(base + L.status);
    job.err_msg = base + L.err;
    CommShared& cs = *(CommShared*)(img + L.cs);
    cs.size = nranks;
    cs.ctx = 1;
    cs.members = nullptr;
    cs.pub = (Pub*)(base + L.pub);
    cs.arrive = (u64*)(base + L.flags);
    cs.mid = cs.arrive + nranks;
    cs.depart = cs.arrive + 2 * (size_t)nranks;
    MPI_Comm_impl* h = (MPI_Comm_impl*)(img + L.handles);
    for (int r = 0; r < nranks; r++) {
        h[r].kind = 1;
        h[r].ctx = 1;
        h[r].size = nranks;
        h[r].rank = r;
        h[r].refcnt = 1;
        h[r].cs = (CommShared*)(base + L.cs);
        h[r].seq = 0;
    }
    DevComm& dc = *(DevComm*)(img + L.dcomm);
    dc.handles = (MPI_Comm_impl*)(base + L.handles);
    dc.size = nranks;
    void** ptrs = (void**)(img + L.ptrs);
    for (int r = 0; r < nranks; r++) {
        ptrs[r] = sendbufs[r];
        ptrs[nranks + r] = recvbufs[r];
    }
    DevDesc& d = *(DevDesc*)(img + L.desc);
    d.op = GPUMPI_COLL_ALLREDUCE;
    d.dtype = dtype;
    d.redop = redop;
    d.root = 0;
    d.count = count;
    d.comm = 0;
    d.esize = es;
    d.algo = 0;
    d.sbufs = (void**)(base + L.ptrs);
    d.rbufs = (void**)(base + L.ptrs) + nranks;
    int* first = (int*)(img + L.first);
    first[0] = 0;
    first[1] = 1;
    cudaStream_t st = (cudaStream_t)stream;
    CK(cudaMemcpyAsync(base, img, L.total, cudaMemcpyHostToDevice, st));
    PlanArgs args;
    args.job = (Job*)(base + L.job);
    args.descs = (const DevDesc*)(base + L.desc);
    args.comm_first = (const int*)(base + L.first);
    args.slot_comm = nullptr;
    args.slot_rank = nullptr;
    args.comms = (const DevComm*)(base + L.dcomm);
    args.ordered = 0;
    args.pad = 0;
    int rc = launch((const void*)gpumpi_plan_kernel, nranks, threads_per_rank, smem, &args, st);
    if (rc) return rc;
    CK(cudaStreamSynchronize(st));
    int status[16];
    CK(cudaMemcpy(status, base + L.status, sizeof(status), cudaMemcpyDeviceToHost));
    if (status[1] != 0) {
        char m[160];
        snprintf(m, sizeof(m), "gpumpi_allreduce_noalloc: device error %d on rank %d", status[1], status[2]);
        set_last_error(m);
        return GPUMPI_EJOB;
    }
    return GPUMPI_OK;
}
