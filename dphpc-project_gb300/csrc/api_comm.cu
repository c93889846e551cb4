// Communicators, groups, Cartesian topologies and user operators (leader side).
// Interfaces as in gpu_libs/gpu_mpi/communicator.cuh:23-49 and group.cuh:21-31.
// Differences from the reference: MPI_Group_rank reports MPI_UNDEFINED through
// its argument instead of its return value (group.cu:110-122), MPI_Comm_rank
// is O(1) instead of a scan of the group, MPI_Barrier works on every
// communicator (mpi.cu:324-331 trapped on anything but WORLD), and the
// Cartesian calls are implemented instead of trapping (communicator.cu:138-146).
#include "rt.cuh"

using namespace gm;

extern __device__ MPI_Group_impl gm_group_world_sentinel;
extern __device__ MPI_Group_impl gm_group_empty_sentinel;
extern __device__ MPI_Comm_impl gm_world_sentinel;

namespace gm {
__device__ int aborted_code();
}

// ---------------------------------------------------------------- communicators
__device__ int MPI_Comm_size(MPI_Comm comm, int* size) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    *size = c->size;
    return MPI_SUCCESS;
}

__device__ int MPI_Comm_rank(MPI_Comm comm, int* rank) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    *rank = c->rank;
    return MPI_SUCCESS;
}

static __device__ int split_call(MPI_Comm_impl* parent, int color, int key, MPI_Comm* newcomm) {
    BlockCtx& b = bctx();
    if (job_aborted(b.job)) return aborted_code();
    Call call;
    call.op = OP_COMM_SPLIT;
    call.a[0] = (u64)parent;
    call.a[1] = (u64)(long long)color;
    call.a[2] = (u64)(long long)key;
    call.a[3] = 0;
    int rc = block_call(call);
    MPI_Comm_impl* h = (MPI_Comm_impl*)call.a[3];
    *newcomm = h ? h : MPI_COMM_NULL;
    return rc;
}

__device__ int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    return split_call(c, color < 0 ? -1 : color, key, newcomm);
}

__device__ int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    int rc = split_call(c, 0, c->rank, newcomm);
    if (rc) return rc;
    MPI_Comm_impl* n = comm_resolve(*newcomm);
    if (n && c->cs->topo_ndims > 0 && n->rank == 0) {
        n->cs->topo_ndims = c->cs->topo_ndims;
        for (int i = 0; i < 8; i++) {
            n->cs->topo_dims[i] = c->cs->topo_dims[i];
            n->cs->topo_periods[i] = c->cs->topo_periods[i];
        }
    }
    if (n && c->cs->topo_ndims > 0) MPI_Barrier(*newcomm);
    return MPI_SUCCESS;
}

static __device__ MPI_Group_impl* group_alloc() {
    RankPriv* p = bctx().priv;
    for (int i = 0; i < MAX_GROUPS; i++) {
        if (p->groups[i].kind == 0) {
            MPI_Group_impl* g = &p->groups[i];
            g->kind = 1;
            g->n = 0;
            g->ranks = nullptr;
            g->refcnt = 1;
            return g;
        }
    }
    return nullptr;
}

// Members of a group as job ranks; identity for WORLD.
struct GroupView {
    int n;
    const int* ranks;
    __device__ int at(int i) const { return ranks ? ranks[i] : i; }
};

static __device__ bool group_view(MPI_Group g, GroupView* v) {
    BlockCtx& b = bctx();
    if (g == &gm_group_world_sentinel) {
        v->n = b.job->nranks;
        v->ranks = nullptr;
        return true;
    }
    if (g == &gm_group_empty_sentinel) {
        v->n = 0;
        v->ranks = nullptr;
        return true;
    }
    RankPriv* p = b.priv;
    if (g < &p->groups[0] || g >= &p->groups[MAX_GROUPS] || g->kind != 1) return false;
    v->n = g->n;
    v->ranks = g->ranks;
    return true;
}

__device__ int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    const int me = comm_world_rank(c, c->rank);
    int pos = -1;
    for (int i = 0; i < v.n; i++)
        if (v.at(i) == me) {
            pos = i;
            break;
        }
    return split_call(c, pos >= 0 ? 0 : -1, pos, newcomm);
}

__device__ int MPI_Comm_free(MPI_Comm* comm) {
    if (!comm) return MPI_ERR_COMM;
    MPI_Comm_impl* c = comm_resolve(*comm);
    if (!c) return MPI_ERR_COMM;
    RankPriv* p = bctx().priv;
    if (c != &p->comms[0] && c != &p->comms[1]) {
        if (--c->refcnt <= 0) c->kind = 0;
        bctx().sc_handle = nullptr;   // the leader paths' cached communicator may be this one
    }
    *comm = MPI_COMM_NULL;
    return MPI_SUCCESS;
}

__device__ int MPI_Comm_group(MPI_Comm comm, MPI_Group* group) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    if (c->cs->members == nullptr && c->size == bctx().job->nranks) {
        *group = MPI_GROUP_WORLD;
        return MPI_SUCCESS;
    }
    MPI_Group_impl* g = group_alloc();
    if (!g) return MPI_ERR_INTERN;
    g->n = c->size;
    g->ranks = (int*)heap_alloc(&bctx().job->heap, sizeof(int) * (c->size ? c->size : 1));
    if (!g->ranks) {
        g->kind = 0;
        return MPI_ERR_NO_MEM;
    }
    for (int i = 0; i < c->size; i++) g->ranks[i] = comm_world_rank(c, i);
    *group = g;
    return MPI_SUCCESS;
}

__device__ int MPI_Comm_compare(MPI_Comm comm1, MPI_Comm comm2, int* result) {
    MPI_Comm_impl* a = comm_resolve(comm1);
    MPI_Comm_impl* b = comm_resolve(comm2);
    if (!a || !b) return MPI_ERR_COMM;
    if (a == b) {
        *result = MPI_IDENT;
        return MPI_SUCCESS;
    }
    if (a->size != b->size) {
        *result = MPI_UNEQUAL;
        return MPI_SUCCESS;
    }
    bool same_order = true, same_set = true;
    for (int i = 0; i < a->size && same_order; i++)
        if (comm_world_rank(a, i) != comm_world_rank(b, i)) same_order = false;
    if (!same_order) {
        for (int i = 0; i < a->size && same_set; i++) {
            int r = comm_world_rank(a, i);
            bool found = false;
            for (int k = 0; k < b->size; k++)
                if (comm_world_rank(b, k) == r) {
                    found = true;
                    break;
                }
            same_set = found;
        }
    }
    *result = same_order ? MPI_CONGRUENT : (same_set ? MPI_SIMILAR : MPI_UNEQUAL);
    return MPI_SUCCESS;
}

__device__ int MPI_Attr_get(MPI_Comm comm, int keyval, void* attribute_val, int* flag) {
    (void)comm;
    (void)keyval;
    (void)attribute_val;
    if (flag) *flag = 0;
    return MPI_SUCCESS;
}

__device__ int MPI_Attr_put(MPI_Comm comm, int keyval, void* attribute_val) {
    (void)comm;
    (void)keyval;
    (void)attribute_val;
    return MPI_SUCCESS;
}

__device__ int MPI_NULL_COPY_FN(MPI_Comm, int, void*, void*, void*, int* flag) {
    if (flag) *flag = 0;
    return MPI_SUCCESS;
}

__device__ int MPI_NULL_DELETE_FN(MPI_Comm, int, void*, void*) { return MPI_SUCCESS; }

__device__ int MPI_Keyval_create(MPI_Copy_function*, MPI_Delete_function*, int* keyval, void*) {
    static __device__ int next_key = 1;
    *keyval = atomicAdd(&next_key, 1);
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- groups
__device__ int MPI_Group_size(MPI_Group group, int* size) {
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    *size = v.n;
    return MPI_SUCCESS;
}

__device__ int MPI_Group_rank(MPI_Group group, int* rank) {
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    const int me = bctx().rank;
    *rank = MPI_UNDEFINED;
    for (int i = 0; i < v.n; i++)
        if (v.at(i) == me) {
            *rank = i;
            break;
        }
    return MPI_SUCCESS;
}

static __device__ int group_from_list(const GroupView& v, int n, const int* idx, MPI_Group* out) {
    MPI_Group_impl* g = group_alloc();
    if (!g) return MPI_ERR_INTERN;
    g->n = n;
    g->ranks = (int*)heap_alloc(&bctx().job->heap, sizeof(int) * (n ? n : 1));
    if (!g->ranks) {
        g->kind = 0;
        return MPI_ERR_NO_MEM;
    }
    for (int i = 0; i < n; i++) {
        if (idx[i] < 0 || idx[i] >= v.n) {
            g->kind = 0;
            heap_free(&bctx().job->heap, g->ranks);
            return MPI_ERR_RANK;
        }
        g->ranks[i] = v.at(idx[i]);
    }
    *out = g;
    return MPI_SUCCESS;
}

__device__ int MPI_Group_incl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup) {
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    return group_from_list(v, n, ranks, newgroup);
}

__device__ int MPI_Group_excl(MPI_Group group, int n, const int ranks[], MPI_Group* newgroup) {
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    int* keep = (int*)heap_alloc(&bctx().job->heap, sizeof(int) * (v.n ? v.n : 1));
    if (!keep) return MPI_ERR_NO_MEM;
    int m = 0;
    for (int i = 0; i < v.n; i++) {
        bool drop = false;
        for (int k = 0; k < n; k++)
            if (ranks[k] == i) drop = true;
        if (!drop) keep[m++] = i;
    }
    int rc = group_from_list(v, m, keep, newgroup);
    heap_free(&bctx().job->heap, keep);
    return rc;
}

// Ranges [first, last, stride] as in MPI; a negative stride walks downwards.
__device__ int MPI_Group_range_incl(MPI_Group group, int n, int ranges[][3], MPI_Group* newgroup) {
    GroupView v;
    if (!group_view(group, &v)) return MPI_ERR_ARG;
    int total = 0;
    for (int i = 0; i < n; i++) {
        int f = ranges[i][0], l = ranges[i][1], s = ranges[i][2];
        if (s == 0) return MPI_ERR_ARG;
        if ((s > 0 && f > l) || (s < 0 && f < l)) continue;
        total += (l - f) / s + 1;
    }
    int* idx = (int*)heap_alloc(&bctx().job->heap, sizeof(int) * (total ? total : 1));
    if (!idx) return MPI_ERR_NO_MEM;
    int m = 0;
    for (int i = 0; i < n; i++) {
        int f = ranges[i][0], l = ranges[i][1], s = ranges[i][2];
        if (s > 0)
            for (int r = f; r <= l; r += s) idx[m++] = r;
        else
            for (int r = f; r >= l; r += s) idx[m++] = r;
    }
    int rc = group_from_list(v, m, idx, newgroup);
    heap_free(&bctx().job->heap, idx);
    return rc;
}

__device__ int MPI_Group_free(MPI_Group* group) {
    if (!group) return MPI_ERR_ARG;
    MPI_Group g = *group;
    if (g == &gm_group_world_sentinel || g == &gm_group_empty_sentinel || g == nullptr) {
        *group = MPI_GROUP_NULL;
        return MPI_SUCCESS;
    }
    GroupView v;
    if (!group_view(g, &v)) return MPI_ERR_ARG;
    if (--g->refcnt <= 0) {
        if (g->ranks) heap_free(&bctx().job->heap, g->ranks);
        g->kind = 0;
    }
    *group = MPI_GROUP_NULL;
    return MPI_SUCCESS;
}

__device__ int MPI_Group_translate_ranks(MPI_Group group1, int n, const int ranks1[],
                                         MPI_Group group2, int ranks2[]) {
    GroupView a, b;
    if (!group_view(group1, &a) || !group_view(group2, &b)) return MPI_ERR_ARG;
    for (int i = 0; i < n; i++) {
        ranks2[i] = MPI_UNDEFINED;
        if (ranks1[i] < 0 || ranks1[i] >= a.n) continue;
        int r = a.at(ranks1[i]);
        for (int k = 0; k < b.n; k++)
            if (b.at(k) == r) {
                ranks2[i] = k;
                break;
            }
    }
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- Cartesian topologies
__device__ int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
    if (ndims <= 0 || ndims > 8) return MPI_ERR_ARG;
    int fixed = 1, nfree = 0;
    for (int i = 0; i < ndims; i++) {
        if (dims[i] < 0) return MPI_ERR_ARG;
        if (dims[i] > 0) fixed *= dims[i];
        else nfree++;
    }
    if (fixed <= 0 || nnodes % fixed) return MPI_ERR_ARG;
    int rem = nnodes / fixed;
    if (nfree == 0) return rem == 1 ? MPI_SUCCESS : MPI_ERR_ARG;
    // Spread the prime factors (largest first) over the free dimensions, each
    // time onto the currently smallest one; then sort the free dims decreasing.
    int f[8];
    for (int i = 0; i < nfree; i++) f[i] = 1;
    int primes[32], np = 0;
    for (int p = 2; p * p <= rem; p++)
        while (rem % p == 0) {
            primes[np++] = p;
            rem /= p;
        }
    if (rem > 1) primes[np++] = rem;
    for (int k = np - 1; k >= 0; k--) {
        int m = 0;
        for (int i = 1; i < nfree; i++)
            if (f[i] < f[m]) m = i;
        f[m] *= primes[k];
    }
    for (int i = 0; i < nfree; i++)
        for (int k = i + 1; k < nfree; k++)
            if (f[k] > f[i]) {
                int t = f[i];
                f[i] = f[k];
                f[k] = t;
            }
    for (int i = 0, k = 0; i < ndims; i++)
        if (dims[i] == 0) dims[i] = f[k++];
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_create(MPI_Comm comm_old, int ndims, const int dims[], const int periods[],
                               int reorder, MPI_Comm* comm_cart) {
    (void)reorder;
    MPI_Comm_impl* c = comm_resolve(comm_old);
    if (!c) return MPI_ERR_COMM;
    if (ndims <= 0 || ndims > 8) return MPI_ERR_ARG;
    int prod = 1;
    for (int i = 0; i < ndims; i++) prod *= dims[i];
    if (prod > c->size) return MPI_ERR_ARG;
    int rc = split_call(c, c->rank < prod ? 0 : -1, c->rank, comm_cart);
    if (rc) return rc;
    MPI_Comm_impl* n = comm_resolve(*comm_cart);
    if (n) {
        if (n->rank == 0) {
            n->cs->topo_ndims = ndims;
            for (int i = 0; i < ndims; i++) {
                n->cs->topo_dims[i] = dims[i];
                n->cs->topo_periods[i] = periods ? periods[i] : 0;
            }
        }
        MPI_Barrier(*comm_cart);
    }
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int coords[]) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    const CommShared* cs = c->cs;
    if (cs->topo_ndims <= 0) return MPI_ERR_ARG;
    int r = rank;
    for (int i = cs->topo_ndims - 1; i >= 0; i--) {
        if (i < maxdims) coords[i] = r % cs->topo_dims[i];
        r /= cs->topo_dims[i];
    }
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_rank(MPI_Comm comm, const int coords[], int* rank) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    const CommShared* cs = c->cs;
    if (cs->topo_ndims <= 0) return MPI_ERR_ARG;
    int r = 0;
    for (int i = 0; i < cs->topo_ndims; i++) {
        int d = cs->topo_dims[i], x = coords[i];
        if (x < 0 || x >= d) {
            if (!cs->topo_periods[i]) return MPI_ERR_RANK;
            x = ((x % d) + d) % d;
        }
        r = r * d + x;
    }
    *rank = r;
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int* rank_source,
                              int* rank_dest) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    const CommShared* cs = c->cs;
    if (cs->topo_ndims <= 0 || direction < 0 || direction >= cs->topo_ndims) return MPI_ERR_ARG;
    int coords[8];
    MPI_Cart_coords(comm, c->rank, 8, coords);
    int d = cs->topo_dims[direction];
    int per = cs->topo_periods[direction];
    int x0 = coords[direction];
    for (int s = 0; s < 2; s++) {
        int x = s == 0 ? x0 - disp : x0 + disp;
        int* out = s == 0 ? rank_source : rank_dest;
        if (x < 0 || x >= d) {
            if (!per) {
                *out = MPI_PROC_NULL;
                continue;
            }
            x = ((x % d) + d) % d;
        }
        coords[direction] = x;
        MPI_Cart_rank(comm, coords, out);
        coords[direction] = x0;
    }
    return MPI_SUCCESS;
}

__device__ int MPI_Cart_sub(MPI_Comm comm, const int remain_dims[], MPI_Comm* comm_new) {
    MPI_Comm_impl* c = comm_resolve(comm);
    if (!c) return MPI_ERR_COMM;
    const CommShared* cs = c->cs;
    if (cs->topo_ndims <= 0) return MPI_ERR_ARG;
    int coords[8];
    MPI_Cart_coords(comm, c->rank, 8, coords);
    int color = 0, key = 0, nd = 0;
    int dims[8], periods[8];
    for (int i = 0; i < cs->topo_ndims; i++) {
        if (remain_dims[i]) {
            key = key * cs->topo_dims[i] + coords[i];
            dims[nd] = cs->topo_dims[i];
            periods[nd] = cs->topo_periods[i];
            nd++;
        } else {
            color = color * cs->topo_dims[i] + coords[i];
        }
    }
    int rc = split_call(c, color, key, comm_new);
    if (rc) return rc;
    MPI_Comm_impl* n = comm_resolve(*comm_new);
    if (n && nd > 0) {
        if (n->rank == 0) {
            n->cs->topo_ndims = nd;
            for (int i = 0; i < nd; i++) {
                n->cs->topo_dims[i] = dims[i];
                n->cs->topo_periods[i] = periods[i];
            }
        }
        MPI_Barrier(*comm_new);
    }
    return MPI_SUCCESS;
}

// ---------------------------------------------------------------- user operators
__device__ int MPI_Op_create(MPI_User_function* user_fn, int commute, MPI_Op* op) {
    MPI_Op_impl* o = (MPI_Op_impl*)heap_alloc(&bctx().job->heap, sizeof(MPI_Op_impl));
    if (!o) return MPI_ERR_NO_MEM;
    o->builtin = -1;
    o->commute = commute;
    o->fn = user_fn;
    *op = o;
    return MPI_SUCCESS;
}

__device__ int MPI_Op_free(MPI_Op* op) {
    if (!op || !*op) return MPI_ERR_OP;
    if ((*op)->builtin < 0) heap_free(&bctx().job->heap, *op);
    *op = MPI_OP_NULL;
    return MPI_SUCCESS;
}
