// Leader-side entry points of the collective API.  Argument checks and the
// staging of local-memory buffers happen here; the schedule itself runs
// block-wide in coll.cu.
#include "rt.cuh"

using namespace gm;

namespace gm {
__device__ int aborted_code();
}

namespace {

// Global-memory view of a caller buffer.  Local-memory buffers are copied to
// the rank's stage area (or the heap when they are large).
struct Staged {
    void* user;
    void* g;
    u64 bytes;
    int heap;
};

__device__ int stage(Staged& s, const void* p, u64 bytes, bool copy_in) {
    s.user = (void*)p;
    s.g = (void*)p;
    s.bytes = bytes;
    s.heap = 0;
    if (p == nullptr || p == MPI_IN_PLACE || bytes == 0 || is_global(p)) return MPI_SUCCESS;
    void* g = bytes <= (u64)STAGE_BYTES ? stage_temp((int)bytes) : nullptr;
    if (!g) {
        g = heap_alloc(&bctx().job->heap, bytes);
        if (!g) return MPI_ERR_NO_MEM;
        s.heap = 1;
    }
    if (copy_in) memcpy(g, p, bytes);
    s.g = g;
    return MPI_SUCCESS;
}

__device__ void unstage(Staged& s, bool copy_out) {
    if (s.g == s.user) return;
    if (copy_out && s.bytes) memcpy(s.user, s.g, s.bytes);
    if (s.heap) heap_free(&bctx().job->heap, s.g);
}

__device__ int enter(MPI_Comm comm, MPI_Comm_impl** c) {
    BlockCtx& b = bctx();
    if (job_aborted(b.job)) return aborted_code();
    *c = comm_resolve(comm);
    if (!*c) return MPI_ERR_COMM;
    return MPI_SUCCESS;
}

__device__ int run(Call& call) {
    int rc = block_call(call);
    return rc;
}

// Resolve the element type and count a builtin or user operator folds over.
__device__ int reduce_type(MPI_Op op, MPI_Datatype dt, int count, CollArgs& a) {
    if (op == nullptr) return MPI_ERR_OP;
    if (count < 0) return MPI_ERR_COUNT;
    int es = dtype_size(dt);
    if (es < 0) return MPI_ERR_TYPE;
    if (op->builtin >= 0) {
        int rc = op_check(op, dt);
        if (rc) return rc;
        int mult;
        int base = dtype_base(dt, &mult);
        a.dtype = (MPI_Datatype)base;
        a.count = (u64)count * mult;
        a.rsize = es / (mult ? mult : 1);
    } else {
        a.dtype = dt;
        a.count = (u64)count;
        a.rsize = es;
    }
    a.op = op;
    a.opi = op->builtin;
    a.ufn = op->fn;
    return MPI_SUCCESS;
}

__device__ u64 extent(const int* counts, const int* displs, int P, long long ucount, int es) {
    u64 m = 0;
    for (int q = 0; q < P; q++) {
        u64 c = counts ? (u64)(long long)counts[q] : (u64)ucount;
        u64 d = displs ? (u64)(long long)displs[q] : (u64)ucount * q;
        if (c && d + c > m) m = d + c;
    }
    return m * (u64)es;
}

}  // namespace

__device__ int MPI_Barrier(MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    Call call;
    call.op = OP_BARRIER;
    call.a[0] = (u64)c;
    return run(call);
}

__device__ int MPI_Bcast(void* buffer, int count, MPI_Datatype datatype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    int es = dtype_size(datatype);
    if (es < 0) return MPI_ERR_TYPE;
    if (count < 0) return MPI_ERR_COUNT;
    if (root < 0 || root >= c->size) return MPI_ERR_ROOT;
    const u64 bytes = (u64)count * es;
    Staged s;
    rc = stage(s, buffer, bytes, c->rank == root);
    if (rc) return rc;
    Call call;
    call.op = OP_BCAST;
    CollArgs& a = call.ca;
    a = CollArgs{};
    a.comm = c;
    a.rbuf = s.g;
    a.count = bytes;
    a.root = root;
    rc = run(call);
    unstage(s, c->rank != root);
    stage_reset();
    return rc;
}

__device__ int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype,
                          MPI_Op op, int root, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    if (root < 0 || root >= c->size) return MPI_ERR_ROOT;
    Call call;
    call.op = OP_REDUCE;
    CollArgs& a = call.ca;
    a = CollArgs{};
    rc = reduce_type(op, datatype, count, a);
    if (rc) return rc;
    const u64 bytes = a.count * a.rsize;
    const bool is_root = c->rank == root;
    Staged ss, rs;
    rc = stage(ss, sendbuf, bytes, true);
    if (rc) return rc;
    rc = stage(rs, is_root ? recvbuf : nullptr, bytes, sendbuf == MPI_IN_PLACE);
    if (rc) return rc;
    a.comm = c;
    a.sbuf = ss.g;
    a.rbuf = rs.g;
    a.root = root;
    rc = run(call);
    unstage(ss, false);
    if (is_root) unstage(rs, true);
    stage_reset();
    return rc;
}

__device__ int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype,
                             MPI_Op op, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    Call call;
    call.op = OP_ALLREDUCE;
    CollArgs& a = call.ca;
    a = CollArgs{};
    rc = reduce_type(op, datatype, count, a);
    if (rc) return rc;
    const u64 bytes = a.count * a.rsize;
    // The reference calls MPI_Allreduce(&x, &x, ...) with aliased buffers
    // (gpu_libs/gpu_mpi/communicator.cu:39); treat that as MPI_IN_PLACE.
    if (sendbuf == recvbuf) sendbuf = MPI_IN_PLACE;
    Staged ss, rs;
    rc = stage(ss, sendbuf, bytes, true);
    if (rc) return rc;
    rc = stage(rs, recvbuf, bytes, sendbuf == MPI_IN_PLACE);
    if (rc) return rc;
    a.comm = c;
    a.sbuf = ss.g;
    a.rbuf = rs.g;
    rc = run(call);
    unstage(ss, false);
    unstage(rs, true);
    stage_reset();
    return rc;
}

__device__ int MPI_Reduce_scatter_block(const void* sendbuf, void* recvbuf, int recvcount,
                                        MPI_Datatype datatype, MPI_Op op, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    Call call;
    call.op = OP_REDUCE_SCATTER_BLOCK;
    CollArgs& a = call.ca;
    a = CollArgs{};
    rc = reduce_type(op, datatype, recvcount, a);
    if (rc) return rc;
    const u64 bytes = a.count * a.rsize;
    Staged ss, rs;
    rc = stage(ss, sendbuf, bytes * c->size, true);
    if (rc) return rc;
    rc = stage(rs, recvbuf, bytes, false);
    if (rc) return rc;
    a.comm = c;
    a.sbuf = ss.g;
    a.rbuf = rs.g;
    rc = run(call);
    unstage(ss, false);
    unstage(rs, true);
    stage_reset();
    return rc;
}

static __device__ int scan_common(const void* sendbuf, void* recvbuf, int count,
                                  MPI_Datatype datatype, MPI_Op op, MPI_Comm comm, int exclusive) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    Call call;
    call.op = OP_SCAN;
    CollArgs& a = call.ca;
    a = CollArgs{};
    rc = reduce_type(op, datatype, count, a);
    if (rc) return rc;
    const u64 bytes = a.count * a.rsize;
    Staged ss, rs;
    rc = stage(ss, sendbuf, bytes, true);
    if (rc) return rc;
    rc = stage(rs, recvbuf, bytes, false);
    if (rc) return rc;
    a.comm = c;
    a.sbuf = ss.g;
    a.rbuf = rs.g;
    a.a0 = exclusive;
    rc = run(call);
    unstage(ss, false);
    unstage(rs, !(exclusive && c->rank == 0));
    stage_reset();
    return rc;
}

__device__ int MPI_Scan(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype,
                        MPI_Op op, MPI_Comm comm) {
    return scan_common(sendbuf, recvbuf, count, datatype, op, comm, 0);
}

__device__ int MPI_Exscan(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype,
                          MPI_Op op, MPI_Comm comm) {
    return scan_common(sendbuf, recvbuf, count, datatype, op, comm, 1);
}

// ---------------------------------------------------------------- gather family
static __device__ int gather_common(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                                    void* recvbuf, const int* recvcounts, const int* displs,
                                    int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    if (root < 0 || root >= c->size) return MPI_ERR_ROOT;
    const bool is_root = c->rank == root;
    const int P = c->size;
    int ss = sendbuf == MPI_IN_PLACE ? 1 : dtype_size(sendtype);
    int rsz = is_root ? dtype_size(recvtype) : 1;
    if (ss < 0 || rsz < 0) return MPI_ERR_TYPE;
    if (sendcount < 0) return MPI_ERR_COUNT;
    Staged sc, sd, sb, rb;
    rc = stage(sc, is_root ? recvcounts : nullptr, sizeof(int) * P, true);
    if (!rc) rc = stage(sd, is_root ? displs : nullptr, sizeof(int) * P, true);
    if (rc) return rc;
    u64 sbytes = sendbuf == MPI_IN_PLACE ? 0 : (u64)sendcount * ss;
    rc = stage(sb, sendbuf, sbytes, true);
    if (rc) return rc;
    u64 rext = is_root ? extent((const int*)sc.g, (const int*)sd.g, P, recvcount, rsz) : 0;
    rc = stage(rb, is_root ? recvbuf : nullptr, rext, sendbuf == MPI_IN_PLACE);
    if (rc) return rc;
    Call call;
    call.op = OP_GATHERV;
    CollArgs& a = call.ca;
    a = CollArgs{};
    a.comm = c;
    a.sbuf = sb.g;
    a.rbuf = rb.g;
    a.rcounts = (const int*)sc.g;
    a.rdispls = (const int*)sd.g;
    a.a0 = recvcount;
    a.a1 = sendcount;
    a.ssize = ss;
    a.rsize = rsz;
    a.root = root;
    rc = run(call);
    unstage(sb, false);
    if (is_root) unstage(rb, true);
    unstage(sc, false);
    unstage(sd, false);
    stage_reset();
    return rc;
}

__device__ int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                          int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm) {
    return gather_common(sendbuf, sendcount, sendtype, recvbuf, nullptr, nullptr, recvcount,
                         recvtype, root, comm);
}

__device__ int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                           void* recvbuf, const int recvcounts[], const int displs[],
                           MPI_Datatype recvtype, int root, MPI_Comm comm) {
    return gather_common(sendbuf, sendcount, sendtype, recvbuf, recvcounts, displs, 0, recvtype,
                         root, comm);
}

static __device__ int scatter_common(const void* sendbuf, const int* sendcounts, const int* displs,
                                     int sendcount, MPI_Datatype sendtype, void* recvbuf,
                                     int recvcount, MPI_Datatype recvtype, int root,
                                     MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    if (root < 0 || root >= c->size) return MPI_ERR_ROOT;
    const bool is_root = c->rank == root;
    const int P = c->size;
    int ss = is_root ? dtype_size(sendtype) : 1;
    int rsz = recvbuf == MPI_IN_PLACE ? 1 : dtype_size(recvtype);
    if (ss < 0 || rsz < 0) return MPI_ERR_TYPE;
    Staged sc, sd, sb, rb;
    rc = stage(sc, is_root ? sendcounts : nullptr, sizeof(int) * P, true);
    if (!rc) rc = stage(sd, is_root ? displs : nullptr, sizeof(int) * P, true);
    if (rc) return rc;
    u64 sext = is_root ? extent((const int*)sc.g, (const int*)sd.g, P, sendcount, ss) : 0;
    rc = stage(sb, is_root ? sendbuf : nullptr, sext, true);
    if (rc) return rc;
    u64 rbytes = recvbuf == MPI_IN_PLACE ? 0 : (u64)recvcount * rsz;
    rc = stage(rb, recvbuf, rbytes, false);
    if (rc) return rc;
    Call call;
    call.op = OP_SCATTERV;
    CollArgs& a = call.ca;
    a = CollArgs{};
    a.comm = c;
    a.sbuf = sb.g;
    a.rbuf = rb.g;
    a.scounts = (const int*)sc.g;
    a.sdispls = (const int*)sd.g;
    a.a0 = recvcount;
    a.a1 = sendcount;
    a.ssize = ss;
    a.rsize = rsz;
    a.root = root;
    rc = run(call);
    unstage(rb, true);
    unstage(sb, false);
    unstage(sc, false);
    unstage(sd, false);
    stage_reset();
    return rc;
}

__device__ int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                           int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm) {
    return scatter_common(sendbuf, nullptr, nullptr, sendcount, sendtype, recvbuf, recvcount,
                          recvtype, root, comm);
}

__device__ int MPI_Scatterv(const void* sendbuf, const int sendcounts[], const int displs[],
                            MPI_Datatype sendtype, void* recvbuf, int recvcount,
                            MPI_Datatype recvtype, int root, MPI_Comm comm) {
    return scatter_common(sendbuf, sendcounts, displs, 0, sendtype, recvbuf, recvcount, recvtype,
                          root, comm);
}

static __device__ int allgather_common(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                                       void* recvbuf, const int* recvcounts, const int* displs,
                                       int recvcount, MPI_Datatype recvtype, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    const int P = c->size;
    int ss = sendbuf == MPI_IN_PLACE ? 1 : dtype_size(sendtype);
    int rsz = dtype_size(recvtype);
    if (ss < 0 || rsz < 0) return MPI_ERR_TYPE;
    Staged sc, sd, sb, rb;
    rc = stage(sc, recvcounts, sizeof(int) * P, true);
    if (!rc) rc = stage(sd, displs, sizeof(int) * P, true);
    if (rc) return rc;
    u64 sbytes = sendbuf == MPI_IN_PLACE ? 0 : (u64)sendcount * ss;
    rc = stage(sb, sendbuf, sbytes, true);
    if (rc) return rc;
    u64 rext = extent((const int*)sc.g, (const int*)sd.g, P, recvcount, rsz);
    rc = stage(rb, recvbuf, rext, sendbuf == MPI_IN_PLACE);
    if (rc) return rc;
    Call call;
    call.op = OP_ALLGATHERV;
    CollArgs& a = call.ca;
    a = CollArgs{};
    a.comm = c;
    a.sbuf = sb.g;
    a.rbuf = rb.g;
    a.rcounts = (const int*)sc.g;
    a.rdispls = (const int*)sd.g;
    a.a0 = recvcount;
    a.a1 = sendcount;
    a.ssize = ss;
    a.rsize = rsz;
    rc = run(call);
    unstage(rb, true);
    unstage(sb, false);
    unstage(sc, false);
    unstage(sd, false);
    stage_reset();
    return rc;
}

// Direct pull allgather; the reference composed Gather + Bcast (gpu_libs/gpu_mpi/mpi.cu:484-493).
__device__ int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                             void* recvbuf, int recvcount, MPI_Datatype recvtype, MPI_Comm comm) {
    return allgather_common(sendbuf, sendcount, sendtype, recvbuf, nullptr, nullptr, recvcount,
                            recvtype, comm);
}

__device__ int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                              void* recvbuf, const int recvcounts[], const int displs[],
                              MPI_Datatype recvtype, MPI_Comm comm) {
    return allgather_common(sendbuf, sendcount, sendtype, recvbuf, recvcounts, displs, 0, recvtype,
                            comm);
}

static __device__ int alltoall_common(const void* sendbuf, const int* sendcounts,
                                      const int* sdispls, int sendcount, MPI_Datatype sendtype,
                                      void* recvbuf, const int* recvcounts, const int* rdispls,
                                      int recvcount, MPI_Datatype recvtype, MPI_Comm comm) {
    MPI_Comm_impl* c;
    int rc = enter(comm, &c);
    if (rc) return rc;
    const int P = c->size;
    int ss = dtype_size(sendtype), rsz = dtype_size(recvtype);
    if (ss < 0 || rsz < 0) return MPI_ERR_TYPE;
    if (sendbuf == MPI_IN_PLACE) return GPUMPI_ERR_UNSUPPORTED;
    Staged scs, sds, rcs, rds, sb, rb;
    rc = stage(scs, sendcounts, sizeof(int) * P, true);
    if (!rc) rc = stage(sds, sdispls, sizeof(int) * P, true);
    if (!rc) rc = stage(rcs, recvcounts, sizeof(int) * P, true);
    if (!rc) rc = stage(rds, rdispls, sizeof(int) * P, true);
    if (rc) return rc;
    u64 sext = extent((const int*)scs.g, (const int*)sds.g, P, sendcount, ss);
    u64 rext = extent((const int*)rcs.g, (const int*)rds.g, P, recvcount, rsz);
    rc = stage(sb, sendbuf, sext, true);
    if (!rc) rc = stage(rb, recvbuf, rext, false);
    if (rc) return rc;
    Call call;
    call.op = OP_ALLTOALLV;
    CollArgs& a = call.ca;
    a = CollArgs{};
    a.comm = c;
    a.sbuf = sb.g;
    a.rbuf = rb.g;
    a.scounts = (const int*)scs.g;
    a.sdispls = (const int*)sds.g;
    a.rcounts = (const int*)rcs.g;
    a.rdispls = (const int*)rds.g;
    a.a0 = recvcount;
    a.a1 = sendcount;
    a.ssize = ss;
    a.rsize = rsz;
    rc = run(call);
    unstage(rb, true);
    unstage(sb, false);
    unstage(scs, false);
    unstage(sds, false);
    unstage(rcs, false);
    unstage(rds, false);
    stage_reset();
    return rc;
}

// Direct pull of every block; the reference posted P-1 Isend/Irecv pairs
// through malloc'd request arrays (gpu_libs/gpu_mpi/mpi.cu:333-408).
__device__ int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype,
                            void* recvbuf, int recvcount, MPI_Datatype recvtype, MPI_Comm comm) {
    return alltoall_common(sendbuf, nullptr, nullptr, sendcount, sendtype, recvbuf, nullptr,
                           nullptr, recvcount, recvtype, comm);
}

__device__ int MPI_Alltoallv(const void* sendbuf, const int sendcounts[], const int sdispls[],
                             MPI_Datatype sendtype, void* recvbuf, const int recvcounts[],
                             const int rdispls[], MPI_Datatype recvtype, MPI_Comm comm) {
    return alltoall_common(sendbuf, sendcounts, sdispls, 0, sendtype, recvbuf, recvcounts,
                           rdispls, 0, recvtype, comm);
}

#define GPUMPI_ATA_DEF(suffix)                                                                     \
    __device__ int MPI_Alltoall_##suffix(const void* sendbuf, int sendcount,                       \
                                         MPI_Datatype sendtype, void* recvbuf, int recvcount,      \
                                         MPI_Datatype recvtype, MPI_Comm comm, bool coalesced) {   \
        (void)coalesced;                                                                           \
        return MPI_Alltoall(sendbuf, sendcount, sendtype, recvbuf, recvcount, recvtype, comm);     \
    }                                                                                              \
    __device__ int MPI_Alltoallv_##suffix(const void* sendbuf, const int sendcounts[],             \
                                          const int sdispls[], MPI_Datatype sendtype,              \
                                          void* recvbuf, const int recvcounts[],                   \
                                          const int rdispls[], MPI_Datatype recvtype,              \
                                          MPI_Comm comm, bool coalesced) {                         \
        (void)coalesced;                                                                           \
        return MPI_Alltoallv(sendbuf, sendcounts, sdispls, sendtype, recvbuf, recvcounts,          \
                             rdispls, recvtype, comm);                                             \
    }
GPUMPI_ATA_DEF(coalesce)
GPUMPI_ATA_DEF(v1)
GPUMPI_ATA_DEF(v2)
GPUMPI_ATA_DEF(v3)
GPUMPI_ATA_DEF(v4)
GPUMPI_ATA_DEF(v5)
GPUMPI_ATA_DEF(v6)
