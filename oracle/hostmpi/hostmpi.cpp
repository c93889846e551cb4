// hostmpi: fork-per-rank MPI over shared memory.  TEST INFRASTRUCTURE ONLY --
// the CPU oracle and CPU baseline of the device runtime (see include/mpi.h).
//
// Transport: every message is copied into a shared-memory pool and appended
// to the receiver's mailbox (eager, two copies), so sends complete at once.
// Matching is in arrival order per receiver and in posting order per receive,
// which gives MPI's non-overtaking rule.  Collectives are built from
// point-to-point messages exactly as the reference builds them
// (gpu_libs/gpu_mpi/mpi.cu), on a separate context so they never match user
// receives.
#include "mpi.h"

#include <errno.h>
#include <pthread.h>
#include <signal.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <time.h>
#include <unistd.h>

#include <algorithm>
#include <vector>

extern "C" int hostmpi_user_main(int argc, char** argv);

namespace {

constexpr int MAXR = 4096;
constexpr size_t POOL_BYTES = (size_t)64 << 30;  // virtual; pages are touched on demand

struct Msg {
    Msg* next;
    int src;
    int tag;
    int ctx;
    int cls;
    size_t bytes;
    char data[1];
};

struct RankBox {
    pthread_mutex_t mu;
    pthread_cond_t cv;
    Msg* head;
    Msg* tail;
    unsigned long gen;
};

struct Shm {
    int nranks;
    volatile int abort_flag;
    pthread_mutex_t pool_mu;
    pthread_cond_t pool_cv;
    char* pool;
    size_t bump;
    size_t end;
    Msg* free_head[64];
    RankBox box[MAXR];
};

Shm* g_shm = nullptr;
int g_rank = 0;
int g_size = 1;
double g_timeout_s = 600.0;
int g_next_ctx = 3;
bool g_initialized = false;
bool g_finalized = false;

double now() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

[[noreturn]] void die(const char* what) {
    fprintf(stderr, "hostmpi rank %d: %s\n", g_rank, what);
    fflush(stderr);
    if (g_shm) g_shm->abort_flag = 1;
    _exit(2);
}

void timed_wait(pthread_cond_t* cv, pthread_mutex_t* mu) {
    timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    ts.tv_nsec += 20 * 1000 * 1000;
    if (ts.tv_nsec >= 1000000000) {
        ts.tv_sec++;
        ts.tv_nsec -= 1000000000;
    }
    pthread_cond_timedwait(cv, mu, &ts);
}

// ------------------------------------------------------------------ pool
Msg* msg_alloc(size_t bytes) {
    size_t need = offsetof(Msg, data) + bytes;
    int cls = 6;
    while (((size_t)1 << cls) < need) cls++;
    Shm* s = g_shm;
    const double t0 = now();
    pthread_mutex_lock(&s->pool_mu);
    for (;;) {
        Msg* m = s->free_head[cls];
        if (m) {
            s->free_head[cls] = m->next;
            pthread_mutex_unlock(&s->pool_mu);
            m->cls = cls;
            return m;
        }
        size_t sz = (size_t)1 << cls;
        if (s->bump + sz <= s->end) {
            m = (Msg*)(s->pool + s->bump);
            s->bump += sz;
            pthread_mutex_unlock(&s->pool_mu);
            m->cls = cls;
            return m;
        }
        if (s->abort_flag) {
            pthread_mutex_unlock(&s->pool_mu);
            die("job aborted");
        }
        if (now() - t0 > g_timeout_s) {
            pthread_mutex_unlock(&s->pool_mu);
            die("message pool exhausted");
        }
        timed_wait(&s->pool_cv, &s->pool_mu);
    }
}

void msg_free(Msg* m) {
    Shm* s = g_shm;
    pthread_mutex_lock(&s->pool_mu);
    m->next = s->free_head[m->cls];
    s->free_head[m->cls] = m;
    pthread_cond_broadcast(&s->pool_cv);
    pthread_mutex_unlock(&s->pool_mu);
}

// ------------------------------------------------------------------ types
struct Derived {
    int base;
    int count;
};
std::vector<Derived> g_types;

int basic_size(int t) {
    switch (t) {
        case MPI_CHAR: case MPI_SIGNED_CHAR: case MPI_UNSIGNED_CHAR: case MPI_C_BOOL: case MPI_INT8_T:
        case MPI_UINT8_T: case MPI_BYTE: case MPI_PACKED: return 1;
        case MPI_SHORT: case MPI_UNSIGNED_SHORT: case MPI_INT16_T: case MPI_UINT16_T: return 2;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: case MPI_WCHAR: case MPI_INT32_T:
        case MPI_UINT32_T: return 4;
        case MPI_LONG: case MPI_LONG_LONG_INT: case MPI_LONG_LONG: case MPI_UNSIGNED_LONG:
        case MPI_UNSIGNED_LONG_LONG: case MPI_DOUBLE: case MPI_LONG_DOUBLE: case MPI_INT64_T:
        case MPI_UINT64_T: case MPI_C_COMPLEX: case MPI_C_FLOAT_COMPLEX: case MPI_2INT:
        case MPI_FLOAT_INT: return 8;
        case MPI_C_DOUBLE_COMPLEX: case MPI_C_LONG_DOUBLE_COMPLEX: case MPI_DOUBLE_INT:
        case MPI_LONG_INT: return 16;
        default: return -1;
    }
}

int type_base(MPI_Datatype t, int* mult) {
    int ti = (int)t;
    if (ti >= 0 && ti < HOSTMPI_NUM_BASIC_TYPES) {
        *mult = 1;
        return ti;
    }
    int k = ti - HOSTMPI_FIRST_DERIVED_TYPE;
    if (k >= 0 && k < (int)g_types.size() && g_types[k].count >= 0) {
        *mult = g_types[k].count;
        return g_types[k].base;
    }
    *mult = 0;
    return -1;
}

int type_size(MPI_Datatype t) {
    int mult;
    int b = type_base(t, &mult);
    return b < 0 ? -1 : basic_size(b) * mult;
}

}  // namespace

// ------------------------------------------------------------------ handles
struct hostmpi_comm {
    int ctx;
    int size;
    int rank;
    std::vector<int> members;  // world ranks
    int topo_ndims;
    int dims[8];
    int periods[8];
};
struct hostmpi_group {
    std::vector<int> members;
    bool builtin;
};
struct hostmpi_op {
    int builtin;
    MPI_User_function* fn;
};
struct hostmpi_request {
    int kind;  // 1 send, 2 recv
    bool done;
    void* buf;
    size_t cap;
    int src;
    int tag;
    int ctx;
    MPI_Status st;
};

static hostmpi_comm g_world_obj, g_self_obj;
static hostmpi_group g_group_world_obj, g_group_empty_obj;
static hostmpi_op g_ops[12] = {{0, nullptr}, {1, nullptr}, {2, nullptr},  {3, nullptr},
                               {4, nullptr}, {5, nullptr}, {6, nullptr},  {7, nullptr},
                               {8, nullptr}, {9, nullptr}, {10, nullptr}, {11, nullptr}};

extern "C" {
MPI_Comm MPI_COMM_WORLD = &g_world_obj;
MPI_Comm MPI_COMM_SELF = &g_self_obj;
MPI_Group MPI_GROUP_WORLD = &g_group_world_obj;
MPI_Group MPI_GROUP_EMPTY = &g_group_empty_obj;
MPI_Op MPI_MAX = &g_ops[0], MPI_MIN = &g_ops[1], MPI_SUM = &g_ops[2], MPI_PROD = &g_ops[3],
       MPI_LAND = &g_ops[4], MPI_BAND = &g_ops[5], MPI_LOR = &g_ops[6], MPI_BOR = &g_ops[7],
       MPI_LXOR = &g_ops[8], MPI_BXOR = &g_ops[9], MPI_MAXLOC = &g_ops[10], MPI_MINLOC = &g_ops[11];
}

namespace {

std::vector<hostmpi_request*> g_posted;  // unmatched receives, in posting order

int coll_ctx(const hostmpi_comm* c) { return c->ctx | 0x40000000; }
int world_of(const hostmpi_comm* c, int r) { return c->members[r]; }

void deliver(int dest_world, int src, int tag, int ctx, const void* buf, size_t bytes) {
    Msg* m = msg_alloc(bytes);
    m->next = nullptr;
    m->src = src;
    m->tag = tag;
    m->ctx = ctx;
    m->bytes = bytes;
    if (bytes) memcpy(m->data, buf, bytes);
    RankBox* b = &g_shm->box[dest_world];
    pthread_mutex_lock(&b->mu);
    if (b->tail) b->tail->next = m;
    else b->head = m;
    b->tail = m;
    b->gen++;
    pthread_cond_broadcast(&b->cv);
    pthread_mutex_unlock(&b->mu);
}

bool matches(const Msg* m, int src, int tag, int ctx) {
    return m->ctx == ctx && (src == MPI_ANY_SOURCE || m->src == src) &&
           (tag == MPI_ANY_TAG || m->tag == tag);
}

// Match posted receives against arrived messages, oldest receive first.
void progress() {
    if (g_posted.empty()) return;
    RankBox* b = &g_shm->box[g_rank];
    std::vector<std::pair<hostmpi_request*, Msg*>> got;
    pthread_mutex_lock(&b->mu);
    for (size_t i = 0; i < g_posted.size();) {
        hostmpi_request* r = g_posted[i];
        Msg* prev = nullptr;
        Msg* m = b->head;
        while (m && !matches(m, r->src, r->tag, r->ctx)) {
            prev = m;
            m = m->next;
        }
        if (m) {
            if (prev) prev->next = m->next;
            else b->head = m->next;
            if (b->tail == m) b->tail = prev;
            got.push_back({r, m});
            g_posted.erase(g_posted.begin() + i);
        } else {
            i++;
        }
    }
    pthread_mutex_unlock(&b->mu);
    for (auto& pr : got) {
        hostmpi_request* r = pr.first;
        Msg* m = pr.second;
        size_t n = m->bytes < r->cap ? m->bytes : r->cap;
        if (n) memcpy(r->buf, m->data, n);
        r->st.MPI_SOURCE = m->src;
        r->st.MPI_TAG = m->tag;
        r->st.MPI_ERROR = m->bytes > r->cap ? MPI_ERR_TRUNCATE : MPI_SUCCESS;
        r->st.hostmpi_count_lo = (int)(n & 0xffffffffu);
        r->st.hostmpi_count_hi = (int)(n >> 32);
        r->done = true;
        msg_free(m);
    }
}

void wait_for(hostmpi_request* r) {
    RankBox* b = &g_shm->box[g_rank];
    const double t0 = now();
    for (;;) {
        pthread_mutex_lock(&b->mu);
        unsigned long gen = b->gen;
        pthread_mutex_unlock(&b->mu);
        progress();
        if (r->done) return;
        if (g_shm->abort_flag) die("job aborted by another rank");
        if (now() - t0 > g_timeout_s) die("receive timed out");
        pthread_mutex_lock(&b->mu);
        if (b->gen == gen) timed_wait(&b->cv, &b->mu);
        pthread_mutex_unlock(&b->mu);
    }
}

hostmpi_request* post_recv(void* buf, size_t cap, int src, int tag, int ctx) {
    hostmpi_request* r = new hostmpi_request();
    r->kind = 2;
    r->done = false;
    r->buf = buf;
    r->cap = cap;
    r->src = src;
    r->tag = tag;
    r->ctx = ctx;
    if (src == MPI_PROC_NULL) {
        r->done = true;
        r->st.MPI_SOURCE = MPI_PROC_NULL;
        r->st.MPI_TAG = MPI_ANY_TAG;
        return r;
    }
    g_posted.push_back(r);
    progress();
    return r;
}

// internal blocking point-to-point on a context
void isend_raw(const hostmpi_comm* c, const void* buf, size_t bytes, int dest, int tag, int ctx) {
    deliver(world_of(c, dest), c->rank, tag, ctx, buf, bytes);
}
void recv_raw(const hostmpi_comm* c, void* buf, size_t bytes, int src, int tag, int ctx) {
    (void)c;
    hostmpi_request* r = post_recv(buf, bytes, src, tag, ctx);
    wait_for(r);
    delete r;
}

// ------------------------------------------------------------------ reductions
template <class T> T f_max(T a, T b) { return a > b ? a : b; }
template <class T> T f_min(T a, T b) { return a > b ? b : a; }

struct CF { float re, im; };
struct CD { double re, im; };
struct I2 { int val, idx; };
struct FI { float val; int idx; };
struct DI { double val; int idx; };
struct LI { long val; int idx; };

template <class T, class F>
void fold(const void* in, void* inout, size_t n, F f) {
    const T* a = (const T*)in;
    T* b = (T*)inout;
    for (size_t i = 0; i < n; i++) b[i] = f(a[i], b[i]);
}

template <class T>
bool int_op(int op, const void* in, void* inout, size_t n) {
    switch (op) {
        case 0: fold<T>(in, inout, n, [](T a, T b) { return f_max(a, b); }); return true;
        case 1: fold<T>(in, inout, n, [](T a, T b) { return f_min(a, b); }); return true;
        case 2: fold<T>(in, inout, n, [](T a, T b) { return (T)(a + b); }); return true;
        case 3: fold<T>(in, inout, n, [](T a, T b) { return (T)(a * b); }); return true;
        case 4: fold<T>(in, inout, n, [](T a, T b) { return (T)(a && b); }); return true;
        case 5: fold<T>(in, inout, n, [](T a, T b) { return (T)(a & b); }); return true;
        case 6: fold<T>(in, inout, n, [](T a, T b) { return (T)(a || b); }); return true;
        case 7: fold<T>(in, inout, n, [](T a, T b) { return (T)(a | b); }); return true;
        case 8: fold<T>(in, inout, n, [](T a, T b) { return (T)((!a) != (!b)); }); return true;
        case 9: fold<T>(in, inout, n, [](T a, T b) { return (T)(a ^ b); }); return true;
    }
    return false;
}

template <class T>
bool float_op(int op, const void* in, void* inout, size_t n) {
    switch (op) {
        case 0: fold<T>(in, inout, n, [](T a, T b) { return f_max(a, b); }); return true;
        case 1: fold<T>(in, inout, n, [](T a, T b) { return f_min(a, b); }); return true;
        case 2: fold<T>(in, inout, n, [](T a, T b) { return (T)(a + b); }); return true;
        case 3: fold<T>(in, inout, n, [](T a, T b) { return (T)(a * b); }); return true;
    }
    return false;
}

template <class T>
void loc_op(int op, const void* in, void* inout, size_t n) {
    if (op == 10)
        fold<T>(in, inout, n, [](T a, T b) {
            if (a.val > b.val) return a;
            if (a.val < b.val) return b;
            return a.idx < b.idx ? a : b;
        });
    else
        fold<T>(in, inout, n, [](T a, T b) {
            if (a.val > b.val) return b;
            if (a.val < b.val) return a;
            return a.idx < b.idx ? a : b;
        });
}

// inout[i] = op(in[i], inout[i]) for count elements of datatype (the
// reference's invokeOperator convention, gpu_libs/gpu_mpi/operators.cu:284-286).
int apply_op(MPI_Op op, MPI_Datatype dt, const void* in, void* inout, int count) {
    if (!op) return MPI_ERR_OP;
    if (op->builtin < 0) {
        int len = count;
        MPI_Datatype d = dt;
        op->fn((void*)in, inout, &len, &d);
        return MPI_SUCCESS;
    }
    int mult;
    int b = type_base(dt, &mult);
    size_t n = (size_t)count * mult;
    int o = op->builtin;
    bool ok = false;
    switch (b) {
        case MPI_SIGNED_CHAR: case MPI_INT8_T: ok = o <= 9 && int_op<signed char>(o, in, inout, n); break;
        case MPI_UNSIGNED_CHAR: case MPI_UINT8_T: ok = o <= 9 && int_op<unsigned char>(o, in, inout, n); break;
        case MPI_BYTE: ok = (o == 5 || o == 7 || o == 9) && int_op<unsigned char>(o, in, inout, n); break;
        case MPI_SHORT: case MPI_INT16_T: ok = o <= 9 && int_op<short>(o, in, inout, n); break;
        case MPI_UNSIGNED_SHORT: case MPI_UINT16_T: ok = o <= 9 && int_op<unsigned short>(o, in, inout, n); break;
        case MPI_INT: case MPI_INT32_T: ok = o <= 9 && int_op<int>(o, in, inout, n); break;
        case MPI_UNSIGNED: case MPI_UINT32_T: ok = o <= 9 && int_op<unsigned>(o, in, inout, n); break;
        case MPI_LONG: case MPI_LONG_LONG_INT: case MPI_LONG_LONG: case MPI_INT64_T:
            ok = o <= 9 && int_op<long long>(o, in, inout, n);
            break;
        case MPI_UNSIGNED_LONG: case MPI_UNSIGNED_LONG_LONG: case MPI_UINT64_T:
            ok = o <= 9 && int_op<unsigned long long>(o, in, inout, n);
            break;
        case MPI_FLOAT: ok = float_op<float>(o, in, inout, n); break;
        case MPI_DOUBLE: case MPI_LONG_DOUBLE: ok = float_op<double>(o, in, inout, n); break;
        case MPI_C_BOOL:
            if (o == 4 || o == 6 || o == 8) ok = int_op<bool>(o, in, inout, n);
            break;
        case MPI_C_COMPLEX: case MPI_C_FLOAT_COMPLEX:
            if (o == 2) fold<CF>(in, inout, n, [](CF a, CF b) { return CF{a.re + b.re, a.im + b.im}; });
            if (o == 3)
                fold<CF>(in, inout, n, [](CF a, CF b) {
                    return CF{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
                });
            ok = o == 2 || o == 3;
            break;
        case MPI_C_DOUBLE_COMPLEX: case MPI_C_LONG_DOUBLE_COMPLEX:
            if (o == 2) fold<CD>(in, inout, n, [](CD a, CD b) { return CD{a.re + b.re, a.im + b.im}; });
            if (o == 3)
                fold<CD>(in, inout, n, [](CD a, CD b) {
                    return CD{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
                });
            ok = o == 2 || o == 3;
            break;
        case MPI_2INT: if (o >= 10) { loc_op<I2>(o, in, inout, n); ok = true; } break;
        case MPI_FLOAT_INT: if (o >= 10) { loc_op<FI>(o, in, inout, n); ok = true; } break;
        case MPI_DOUBLE_INT: if (o >= 10) { loc_op<DI>(o, in, inout, n); ok = true; } break;
        case MPI_LONG_INT: if (o >= 10) { loc_op<LI>(o, in, inout, n); ok = true; } break;
        default: break;
    }
    return ok ? MPI_SUCCESS : MPI_ERR_OP;
}

hostmpi_comm* new_comm(int ctx, const std::vector<int>& members) {
    hostmpi_comm* c = new hostmpi_comm();
    c->ctx = ctx;
    c->members = members;
    c->size = (int)members.size();
    c->rank = -1;
    for (int i = 0; i < c->size; i++)
        if (members[i] == g_rank) c->rank = i;
    c->topo_ndims = 0;
    return c;
}

// Context id agreed on by max-reduction over the parent, as in
// gpu_libs/gpu_mpi/communicator.cu:37-46.
int new_context(MPI_Comm comm) {
    int mine = g_next_ctx, agreed = 0;
    MPI_Allreduce(&mine, &agreed, 1, MPI_INT, MPI_MAX, comm);
    g_next_ctx = agreed + 1;
    return agreed;
}

}  // namespace

// ------------------------------------------------------------------ API
extern "C" {

int MPI_Init(int*, char***) {
    g_initialized = true;
    return MPI_SUCCESS;
}
int MPI_Init_thread(int* a, char*** b, int, int* provided) {
    if (provided) *provided = MPI_THREAD_SINGLE;
    return MPI_Init(a, b);
}
int MPI_Initialized(int* flag) {
    *flag = g_initialized;
    return MPI_SUCCESS;
}
int MPI_Finalize(void) {
    MPI_Barrier(MPI_COMM_WORLD);
    g_finalized = true;
    return MPI_SUCCESS;
}
int MPI_Finalized(int* flag) {
    *flag = g_finalized;
    return MPI_SUCCESS;
}
int MPI_Abort(MPI_Comm, int errorcode) {
    fflush(stdout);
    fprintf(stderr, "hostmpi rank %d: MPI_Abort(%d)\n", g_rank, errorcode);
    fflush(stderr);
    g_shm->abort_flag = 1;
    _exit(errorcode ? errorcode : 1);
}
int MPI_Get_processor_name(char* name, int* len) {
    gethostname(name, MPI_MAX_PROCESSOR_NAME);
    *len = (int)strlen(name);
    return MPI_SUCCESS;
}
int MPI_Error_string(int code, char* s, int* len) {
    *len = snprintf(s, MPI_MAX_ERROR_STRING, "MPI error %d", code);
    return MPI_SUCCESS;
}
double MPI_Wtime(void) { return now(); }
double MPI_Wtick(void) { return 1e-9; }

int MPI_Type_size(MPI_Datatype t, int* size) {
    int s = type_size(t);
    if (s < 0) return MPI_ERR_TYPE;
    *size = s;
    return MPI_SUCCESS;
}
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* nt) {
    int mult;
    int b = type_base(old, &mult);
    if (b < 0) return MPI_ERR_TYPE;
    g_types.push_back({b, count * mult});
    *nt = (MPI_Datatype)(HOSTMPI_FIRST_DERIVED_TYPE + (int)g_types.size() - 1);
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype* t) { return type_size(*t) < 0 ? MPI_ERR_TYPE : MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype* t) {
    int k = (int)*t - HOSTMPI_FIRST_DERIVED_TYPE;
    if (k >= 0 && k < (int)g_types.size()) g_types[k].count = -1;
    *t = MPI_DATATYPE_NULL;
    return MPI_SUCCESS;
}
int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* count) {
    int s = type_size(t);
    if (s < 0) return MPI_ERR_TYPE;
    size_t bytes = ((size_t)(unsigned)st->hostmpi_count_hi << 32) | (unsigned)st->hostmpi_count_lo;
    *count = s == 0 ? 0 : (bytes % s ? MPI_UNDEFINED : (int)(bytes / s));
    return MPI_SUCCESS;
}

int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request* req) {
    int es = type_size(t);
    if (es < 0) return MPI_ERR_TYPE;
    hostmpi_request* r = new hostmpi_request();
    r->kind = 1;
    r->done = true;
    memset(&r->st, 0, sizeof(r->st));
    if (dest != MPI_PROC_NULL) deliver(world_of(comm, dest), comm->rank, tag, comm->ctx, buf, (size_t)count * es);
    *req = r;
    return MPI_SUCCESS;
}
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm,
              MPI_Request* req) {
    int es = type_size(t);
    if (es < 0) return MPI_ERR_TYPE;
    *req = post_recv(buf, (size_t)count * es, source, tag, comm->ctx);
    return MPI_SUCCESS;
}
int MPI_Wait(MPI_Request* req, MPI_Status* st) {
    if (!req || !*req) {
        if (st) {
            st->MPI_SOURCE = MPI_ANY_SOURCE;
            st->MPI_TAG = MPI_ANY_TAG;
            st->MPI_ERROR = 0;
            st->hostmpi_count_lo = st->hostmpi_count_hi = 0;
        }
        return MPI_SUCCESS;
    }
    hostmpi_request* r = *req;
    if (!r->done) wait_for(r);
    int err = r->kind == 2 ? r->st.MPI_ERROR : MPI_SUCCESS;
    if (st && r->kind == 2) *st = r->st;
    delete r;
    *req = MPI_REQUEST_NULL;
    return err;
}
int MPI_Test(MPI_Request* req, int* flag, MPI_Status* st) {
    if (!req || !*req) {
        *flag = 1;
        return MPI_SUCCESS;
    }
    progress();
    if (!(*req)->done) {
        *flag = 0;
        return MPI_SUCCESS;
    }
    *flag = 1;
    return MPI_Wait(req, st);
}
int MPI_Waitall(int n, MPI_Request reqs[], MPI_Status* sts) {
    int first = 0;
    for (int i = 0; i < n; i++) {
        int rc = MPI_Wait(&reqs[i], sts ? &sts[i] : nullptr);
        if (rc && !first) first = rc;
    }
    return first;
}
int MPI_Testall(int n, MPI_Request reqs[], int* flag, MPI_Status sts[]) {
    progress();
    for (int i = 0; i < n; i++)
        if (reqs[i] && !reqs[i]->done) {
            *flag = 0;
            return MPI_SUCCESS;
        }
    *flag = 1;
    return MPI_Waitall(n, reqs, sts);
}
int MPI_Waitany(int n, MPI_Request reqs[], int* index, MPI_Status* st) {
    const double t0 = now();
    for (;;) {
        progress();
        int active = 0;
        for (int i = 0; i < n; i++) {
            if (!reqs[i]) continue;
            active = 1;
            if (reqs[i]->done) {
                *index = i;
                return MPI_Wait(&reqs[i], st);
            }
        }
        if (!active) {
            *index = MPI_UNDEFINED;
            return MPI_SUCCESS;
        }
        if (now() - t0 > g_timeout_s) die("MPI_Waitany timed out");
        usleep(50);
    }
}
int MPI_Waitsome(int n, MPI_Request reqs[], int* outcount, int idx[], MPI_Status sts[]) {
    const double t0 = now();
    for (;;) {
        progress();
        int active = 0, k = 0;
        for (int i = 0; i < n; i++) {
            if (!reqs[i]) continue;
            active = 1;
            if (reqs[i]->done) {
                idx[k] = i;
                MPI_Wait(&reqs[i], sts ? &sts[k] : nullptr);
                k++;
            }
        }
        if (!active) {
            *outcount = MPI_UNDEFINED;
            return MPI_SUCCESS;
        }
        if (k) {
            *outcount = k;
            return MPI_SUCCESS;
        }
        if (now() - t0 > g_timeout_s) die("MPI_Waitsome timed out");
        usleep(50);
    }
}
int MPI_Request_free(MPI_Request* req) { return MPI_Wait(req, nullptr); }
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm) {
    MPI_Request r;
    MPI_Isend(buf, count, t, dest, tag, comm, &r);
    return MPI_Wait(&r, nullptr);
}
int MPI_Ssend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm) {
    return MPI_Send(buf, count, t, dest, tag, comm);
}
int MPI_Recv(void* buf, int count, MPI_Datatype t, int source, int tag, MPI_Comm comm,
             MPI_Status* st) {
    MPI_Request r;
    int rc = MPI_Irecv(buf, count, t, source, tag, comm, &r);
    if (rc) return rc;
    return MPI_Wait(&r, st);
}
int MPI_Sendrecv(const void* sb, int sc, MPI_Datatype st_, int dest, int stag, void* rb, int rc_,
                 MPI_Datatype rt, int source, int rtag, MPI_Comm comm, MPI_Status* st) {
    MPI_Request r, s;
    MPI_Irecv(rb, rc_, rt, source, rtag, comm, &r);
    MPI_Isend(sb, sc, st_, dest, stag, comm, &s);
    MPI_Wait(&s, nullptr);
    return MPI_Wait(&r, st);
}
int MPI_Sendrecv_replace(void* buf, int count, MPI_Datatype t, int dest, int stag, int source,
                         int rtag, MPI_Comm comm, MPI_Status* st) {
    size_t bytes = (size_t)count * type_size(t);
    std::vector<char> tmp((char*)buf, (char*)buf + bytes);
    return MPI_Sendrecv(tmp.data(), count, t, dest, stag, buf, count, t, source, rtag, comm, st);
}
int MPI_Iprobe(int source, int tag, MPI_Comm comm, int* flag, MPI_Status* st) {
    progress();
    RankBox* b = &g_shm->box[g_rank];
    pthread_mutex_lock(&b->mu);
    Msg* m = b->head;
    while (m && !matches(m, source, tag, comm->ctx)) m = m->next;
    if (m && st) {
        st->MPI_SOURCE = m->src;
        st->MPI_TAG = m->tag;
        st->MPI_ERROR = 0;
        st->hostmpi_count_lo = (int)(m->bytes & 0xffffffffu);
        st->hostmpi_count_hi = (int)(m->bytes >> 32);
    }
    *flag = m != nullptr;
    pthread_mutex_unlock(&b->mu);
    return MPI_SUCCESS;
}
int MPI_Probe(int source, int tag, MPI_Comm comm, MPI_Status* st) {
    const double t0 = now();
    for (;;) {
        int flag = 0;
        MPI_Iprobe(source, tag, comm, &flag, st);
        if (flag) return MPI_SUCCESS;
        if (g_shm->abort_flag) die("job aborted by another rank");
        if (now() - t0 > g_timeout_s) die("MPI_Probe timed out");
        usleep(20);
    }
}

// ---- collectives: the reference's flat, root-serial algorithms
int MPI_Barrier(MPI_Comm c) {
    const int ctx = coll_ctx(c);
    if (c->rank == 0) {
        for (int q = 1; q < c->size; q++) recv_raw(c, nullptr, 0, q, 1, ctx);
        for (int q = 1; q < c->size; q++) isend_raw(c, nullptr, 0, q, 2, ctx);
    } else {
        isend_raw(c, nullptr, 0, 0, 1, ctx);
        recv_raw(c, nullptr, 0, 0, 2, ctx);
    }
    return MPI_SUCCESS;
}

int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm c) {
    size_t bytes = (size_t)count * type_size(t);
    const int ctx = coll_ctx(c);
    if (c->rank == root) {
        for (int q = 0; q < c->size; q++)
            if (q != root) isend_raw(c, buf, bytes, q, 3, ctx);
    } else {
        recv_raw(c, buf, bytes, root, 3, ctx);
    }
    return MPI_SUCCESS;
}

// Root receives every contribution, then folds in rank order:
// acc = x_0; acc = op(x_q, acc) for q = 1..P-1 (gpu_libs/gpu_mpi/mpi.cu:200-225).
int MPI_Reduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) {
    const int es = type_size(t);
    if (es < 0) return MPI_ERR_TYPE;
    const size_t bytes = (size_t)count * es;
    const int ctx = coll_ctx(c);
    if (c->rank != root) {
        isend_raw(c, sb, bytes, root, 4, ctx);
        return MPI_SUCCESS;
    }
    const int P = c->size;
    std::vector<char> all((size_t)P * bytes + 1);
    for (int q = 0; q < P; q++) {
        char* dst = all.data() + (size_t)q * bytes;
        if (q == root) memcpy(dst, sb == MPI_IN_PLACE ? rb : sb, bytes);
        else recv_raw(c, dst, bytes, q, 4, ctx);
    }
    memcpy(rb, all.data(), bytes);
    for (int q = 1; q < P; q++) {
        int rc = apply_op(op, t, all.data() + (size_t)q * bytes, rb, count);
        if (rc) return rc;
    }
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    if (sb == rb) sb = MPI_IN_PLACE;
    const size_t bytes = (size_t)count * type_size(t);
    std::vector<char> in;
    if (sb == MPI_IN_PLACE) {
        in.assign((char*)rb, (char*)rb + bytes);
        sb = in.data();
    }
    int rc = MPI_Reduce(sb, rb, count, t, op, 0, c);
    if (rc) return rc;
    return MPI_Bcast(rb, count, t, 0, c);
}

int MPI_Reduce_scatter_block(const void* sb, void* rb, int rcount, MPI_Datatype t, MPI_Op op,
                             MPI_Comm c) {
    const size_t bytes = (size_t)rcount * type_size(t);
    std::vector<char> full(bytes * c->size + 1);
    int rc = MPI_Reduce(sb, full.data(), rcount * c->size, t, op, 0, c);
    if (rc) return rc;
    return MPI_Scatter(full.data(), rcount, t, rb, rcount, t, 0, c);
}

static int scan_impl(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c,
                     bool exclusive) {
    const size_t bytes = (size_t)count * type_size(t);
    const int ctx = coll_ctx(c);
    std::vector<char> acc(bytes + 1);
    if (c->rank == 0) {
        memcpy(acc.data(), sb, bytes);
        if (!exclusive) memcpy(rb, sb, bytes);
    } else {
        recv_raw(c, acc.data(), bytes, c->rank - 1, 5, ctx);
        if (exclusive) memcpy(rb, acc.data(), bytes);
        int rc = apply_op(op, t, sb, acc.data(), count);
        if (rc) return rc;
        if (!exclusive) memcpy(rb, acc.data(), bytes);
    }
    if (c->rank + 1 < c->size) isend_raw(c, acc.data(), bytes, c->rank + 1, 5, ctx);
    return MPI_SUCCESS;
}
int MPI_Scan(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    return scan_impl(sb, rb, count, t, op, c, false);
}
int MPI_Exscan(const void* sb, void* rb, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c) {
    return scan_impl(sb, rb, count, t, op, c, true);
}

int MPI_Gatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int rcounts[],
                const int displs[], MPI_Datatype rt, int root, MPI_Comm c) {
    const int ctx = coll_ctx(c);
    if (c->rank != root) {
        isend_raw(c, sb, (size_t)sc * type_size(st), root, 6, ctx);
        return MPI_SUCCESS;
    }
    const int rs = type_size(rt);
    for (int q = 0; q < c->size; q++) {
        char* dst = (char*)rb + (size_t)displs[q] * rs;
        size_t n = (size_t)rcounts[q] * rs;
        if (q == root) {
            if (sb != MPI_IN_PLACE) memcpy(dst, sb, std::min(n, (size_t)sc * type_size(st)));
        } else {
            recv_raw(c, dst, n, q, 6, ctx);
        }
    }
    return MPI_SUCCESS;
}
int MPI_Gather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, int root,
               MPI_Comm c) {
    std::vector<int> counts(c->size, rc), displs(c->size);
    for (int q = 0; q < c->size; q++) displs[q] = q * rc;
    return MPI_Gatherv(sb, sc, st, rb, counts.data(), displs.data(), rt, root, c);
}
int MPI_Scatterv(const void* sb, const int scounts[], const int displs[], MPI_Datatype st, void* rb,
                 int rc, MPI_Datatype rt, int root, MPI_Comm c) {
    const int ctx = coll_ctx(c);
    const size_t rbytes = (size_t)rc * type_size(rt);
    if (c->rank != root) {
        recv_raw(c, rb, rbytes, root, 7, ctx);
        return MPI_SUCCESS;
    }
    const int ss = type_size(st);
    for (int q = 0; q < c->size; q++) {
        const char* src = (const char*)sb + (size_t)displs[q] * ss;
        size_t n = (size_t)scounts[q] * ss;
        if (q == root) {
            if (rb != MPI_IN_PLACE) memcpy(rb, src, std::min(n, rbytes));
        } else {
            isend_raw(c, src, n, q, 7, ctx);
        }
    }
    return MPI_SUCCESS;
}
int MPI_Scatter(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, int root,
                MPI_Comm c) {
    std::vector<int> counts(c->size, sc), displs(c->size);
    for (int q = 0; q < c->size; q++) displs[q] = q * sc;
    return MPI_Scatterv(sb, counts.data(), displs.data(), st, rb, rc, rt, root, c);
}
int MPI_Allgatherv(const void* sb, int sc, MPI_Datatype st, void* rb, const int rcounts[],
                   const int displs[], MPI_Datatype rt, MPI_Comm c) {
    const int rs = type_size(rt);
    if (sb == MPI_IN_PLACE && c->rank != 0) {
        sb = (const char*)rb + (size_t)displs[c->rank] * rs;
        sc = rcounts[c->rank];
        st = rt;
    }
    int rc = MPI_Gatherv(sb, sc, st, rb, rcounts, displs, rt, 0, c);
    if (rc) return rc;
    int ext = 0;
    for (int q = 0; q < c->size; q++) ext = std::max(ext, displs[q] + rcounts[q]);
    return MPI_Bcast(rb, ext, rt, 0, c);
}
int MPI_Allgather(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt,
                  MPI_Comm c) {
    std::vector<int> counts(c->size, rc), displs(c->size);
    for (int q = 0; q < c->size; q++) displs[q] = q * rc;
    return MPI_Allgatherv(sb, sc, st, rb, counts.data(), displs.data(), rt, c);
}
int MPI_Alltoallv(const void* sb, const int scounts[], const int sdispls[], MPI_Datatype st, void* rb,
                  const int rcounts[], const int rdispls[], MPI_Datatype rt, MPI_Comm c) {
    const int ctx = coll_ctx(c);
    const int ss = type_size(st), rs = type_size(rt);
    std::vector<hostmpi_request*> rr;
    for (int q = 0; q < c->size; q++)
        if (q != c->rank) isend_raw(c, (const char*)sb + (size_t)sdispls[q] * ss, (size_t)scounts[q] * ss, q, 8, ctx);
    for (int q = 0; q < c->size; q++)
        if (q != c->rank)
            rr.push_back(post_recv((char*)rb + (size_t)rdispls[q] * rs, (size_t)rcounts[q] * rs, q, 8, ctx));
    memcpy((char*)rb + (size_t)rdispls[c->rank] * rs, (const char*)sb + (size_t)sdispls[c->rank] * ss,
           std::min((size_t)rcounts[c->rank] * rs, (size_t)scounts[c->rank] * ss));
    for (auto* r : rr) {
        wait_for(r);
        delete r;
    }
    return MPI_SUCCESS;
}
int MPI_Alltoall(const void* sb, int sc, MPI_Datatype st, void* rb, int rc, MPI_Datatype rt, MPI_Comm c) {
    std::vector<int> scs(c->size, sc), sds(c->size), rcs(c->size, rc), rds(c->size);
    for (int q = 0; q < c->size; q++) {
        sds[q] = q * sc;
        rds[q] = q * rc;
    }
    return MPI_Alltoallv(sb, scs.data(), sds.data(), st, rb, rcs.data(), rds.data(), rt, c);
}

// ---- communicators and groups
int MPI_Comm_size(MPI_Comm c, int* s) {
    if (!c) return MPI_ERR_COMM;
    *s = c->size;
    return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm c, int* r) {
    if (!c) return MPI_ERR_COMM;
    *r = c->rank;
    return MPI_SUCCESS;
}
int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* out) {
    int mine[2] = {color, key};
    std::vector<int> all(2 * (size_t)c->size);
    MPI_Allgather(mine, 2, MPI_INT, all.data(), 2, MPI_INT, c);
    int ctx = new_context(c);
    if (color < 0) {
        *out = MPI_COMM_NULL;
        return MPI_SUCCESS;
    }
    std::vector<std::pair<int, int>> kr;
    for (int q = 0; q < c->size; q++)
        if (all[2 * q] == color) kr.push_back({all[2 * q + 1], q});
    std::sort(kr.begin(), kr.end());
    std::vector<int> members;
    for (auto& p : kr) members.push_back(world_of(c, p.second));
    *out = new_comm(ctx, members);
    return MPI_SUCCESS;
}
int MPI_Comm_dup(MPI_Comm c, MPI_Comm* out) {
    int ctx = new_context(c);
    hostmpi_comm* n = new_comm(ctx, c->members);
    n->topo_ndims = c->topo_ndims;
    memcpy(n->dims, c->dims, sizeof(n->dims));
    memcpy(n->periods, c->periods, sizeof(n->periods));
    *out = n;
    return MPI_SUCCESS;
}
int MPI_Comm_create(MPI_Comm c, MPI_Group g, MPI_Comm* out) {
    int ctx = new_context(c);
    bool in = false;
    for (int r : g->members)
        if (r == g_rank) in = true;
    *out = in ? new_comm(ctx, g->members) : MPI_COMM_NULL;
    return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm* c) {
    if (*c != MPI_COMM_WORLD && *c != MPI_COMM_SELF) delete *c;
    *c = MPI_COMM_NULL;
    return MPI_SUCCESS;
}
int MPI_Comm_group(MPI_Comm c, MPI_Group* g) {
    hostmpi_group* n = new hostmpi_group();
    n->members = c->members;
    n->builtin = false;
    *g = n;
    return MPI_SUCCESS;
}
int MPI_Comm_compare(MPI_Comm a, MPI_Comm b, int* result) {
    if (a == b) *result = MPI_IDENT;
    else if (a->members == b->members) *result = MPI_CONGRUENT;
    else {
        std::vector<int> x = a->members, y = b->members;
        std::sort(x.begin(), x.end());
        std::sort(y.begin(), y.end());
        *result = x == y ? MPI_SIMILAR : MPI_UNEQUAL;
    }
    return MPI_SUCCESS;
}
int MPI_Group_incl(MPI_Group g, int n, const int ranks[], MPI_Group* out) {
    hostmpi_group* ng = new hostmpi_group();
    ng->builtin = false;
    for (int i = 0; i < n; i++) ng->members.push_back(g->members[ranks[i]]);
    *out = ng;
    return MPI_SUCCESS;
}
int MPI_Group_excl(MPI_Group g, int n, const int ranks[], MPI_Group* out) {
    hostmpi_group* ng = new hostmpi_group();
    ng->builtin = false;
    for (int i = 0; i < (int)g->members.size(); i++) {
        bool drop = false;
        for (int k = 0; k < n; k++)
            if (ranks[k] == i) drop = true;
        if (!drop) ng->members.push_back(g->members[i]);
    }
    *out = ng;
    return MPI_SUCCESS;
}
int MPI_Group_range_incl(MPI_Group g, int n, int ranges[][3], MPI_Group* out) {
    hostmpi_group* ng = new hostmpi_group();
    ng->builtin = false;
    for (int i = 0; i < n; i++) {
        int f = ranges[i][0], l = ranges[i][1], s = ranges[i][2];
        if (s > 0)
            for (int r = f; r <= l; r += s) ng->members.push_back(g->members[r]);
        else if (s < 0)
            for (int r = f; r >= l; r += s) ng->members.push_back(g->members[r]);
    }
    *out = ng;
    return MPI_SUCCESS;
}
int MPI_Group_free(MPI_Group* g) {
    if (*g && !(*g)->builtin) delete *g;
    *g = MPI_GROUP_NULL;
    return MPI_SUCCESS;
}
int MPI_Group_size(MPI_Group g, int* s) {
    *s = (int)g->members.size();
    return MPI_SUCCESS;
}
int MPI_Group_rank(MPI_Group g, int* r) {
    *r = MPI_UNDEFINED;
    for (int i = 0; i < (int)g->members.size(); i++)
        if (g->members[i] == g_rank) *r = i;
    return MPI_SUCCESS;
}
int MPI_Group_translate_ranks(MPI_Group a, int n, const int r1[], MPI_Group b, int r2[]) {
    for (int i = 0; i < n; i++) {
        r2[i] = MPI_UNDEFINED;
        int w = a->members[r1[i]];
        for (int k = 0; k < (int)b->members.size(); k++)
            if (b->members[k] == w) r2[i] = k;
    }
    return MPI_SUCCESS;
}
int MPI_Dims_create(int nnodes, int ndims, int dims[]) {
    int fixed = 1, nfree = 0;
    for (int i = 0; i < ndims; i++) {
        if (dims[i] > 0) fixed *= dims[i];
        else nfree++;
    }
    if (fixed <= 0 || nnodes % fixed) return MPI_ERR_ARG;
    int rem = nnodes / fixed;
    if (!nfree) return rem == 1 ? MPI_SUCCESS : MPI_ERR_ARG;
    std::vector<int> f(nfree, 1), primes;
    for (int p = 2; p * p <= rem; p++)
        while (rem % p == 0) {
            primes.push_back(p);
            rem /= p;
        }
    if (rem > 1) primes.push_back(rem);
    for (int k = (int)primes.size() - 1; k >= 0; k--) {
        int m = 0;
        for (int i = 1; i < nfree; i++)
            if (f[i] < f[m]) m = i;
        f[m] *= primes[k];
    }
    std::sort(f.begin(), f.end(), [](int a, int b) { return a > b; });
    for (int i = 0, k = 0; i < ndims; i++)
        if (dims[i] == 0) dims[i] = f[k++];
    return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm old, int nd, const int dims[], const int periods[], int, MPI_Comm* out) {
    int prod = 1;
    for (int i = 0; i < nd; i++) prod *= dims[i];
    int rc = MPI_Comm_split(old, old->rank < prod ? 0 : MPI_UNDEFINED, old->rank, out);
    if (rc || !*out) return rc;
    (*out)->topo_ndims = nd;
    for (int i = 0; i < nd; i++) {
        (*out)->dims[i] = dims[i];
        (*out)->periods[i] = periods ? periods[i] : 0;
    }
    return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm c, int rank, int maxdims, int coords[]) {
    int r = rank;
    for (int i = c->topo_ndims - 1; i >= 0; i--) {
        if (i < maxdims) coords[i] = r % c->dims[i];
        r /= c->dims[i];
    }
    return MPI_SUCCESS;
}
int MPI_Cart_rank(MPI_Comm c, const int coords[], int* rank) {
    int r = 0;
    for (int i = 0; i < c->topo_ndims; i++) {
        int d = c->dims[i], x = coords[i];
        if (x < 0 || x >= d) {
            if (!c->periods[i]) return MPI_ERR_RANK;
            x = ((x % d) + d) % d;
        }
        r = r * d + x;
    }
    *rank = r;
    return MPI_SUCCESS;
}
int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int* src, int* dst) {
    int coords[8];
    MPI_Cart_coords(c, c->rank, 8, coords);
    int d = c->dims[dir], x0 = coords[dir];
    for (int s = 0; s < 2; s++) {
        int x = s == 0 ? x0 - disp : x0 + disp;
        int* out = s == 0 ? src : dst;
        if (x < 0 || x >= d) {
            if (!c->periods[dir]) {
                *out = MPI_PROC_NULL;
                continue;
            }
            x = ((x % d) + d) % d;
        }
        coords[dir] = x;
        MPI_Cart_rank(c, coords, out);
        coords[dir] = x0;
    }
    return MPI_SUCCESS;
}
int MPI_Cart_sub(MPI_Comm c, const int remain[], MPI_Comm* out) {
    int coords[8];
    MPI_Cart_coords(c, c->rank, 8, coords);
    int color = 0, key = 0, nd = 0, dims[8], per[8];
    for (int i = 0; i < c->topo_ndims; i++) {
        if (remain[i]) {
            key = key * c->dims[i] + coords[i];
            dims[nd] = c->dims[i];
            per[nd] = c->periods[i];
            nd++;
        } else {
            color = color * c->dims[i] + coords[i];
        }
    }
    int rc = MPI_Comm_split(c, color, key, out);
    if (rc || !*out) return rc;
    (*out)->topo_ndims = nd;
    for (int i = 0; i < nd; i++) {
        (*out)->dims[i] = dims[i];
        (*out)->periods[i] = per[i];
    }
    return MPI_SUCCESS;
}
int MPI_Attr_get(MPI_Comm, int, void*, int* flag) {
    *flag = 0;
    return MPI_SUCCESS;
}
int MPI_Attr_put(MPI_Comm, int, void*) { return MPI_SUCCESS; }
int MPI_Keyval_create(MPI_Copy_function*, MPI_Delete_function*, int* keyval, void*) {
    static int next = 1;
    *keyval = next++;
    return MPI_SUCCESS;
}
int MPI_Op_create(MPI_User_function* fn, int, MPI_Op* op) {
    *op = new hostmpi_op{-1, fn};
    return MPI_SUCCESS;
}
int MPI_Op_free(MPI_Op* op) {
    if (*op && (*op)->builtin < 0) delete *op;
    *op = MPI_OP_NULL;
    return MPI_SUCCESS;
}

}  // extern "C"

// ------------------------------------------------------------------ launcher
// Same command line as the GPU launcher: program arguments, "---gpumpi",
// then -n N (or -g G -b B).  Options that only concern the GPU are accepted
// and ignored.
int main(int argc, char** argv) {
    int pos = -1;
    for (int i = 0; i < argc; i++)
        if (strcmp(argv[i], "---gpumpi") == 0) pos = i;
    int n = 0, g = 0, b = 0;
    double max_seconds = 900.0;
    if (pos >= 0) {
        for (int i = pos + 1; i < argc; i++) {
            const char* a = argv[i];
            const char* v = i + 1 < argc ? argv[i + 1] : "0";
            if (!strcmp(a, "-n") || !strcmp(a, "--numProcs")) n = atoi(v), i++;
            else if (!strcmp(a, "-g") || !strcmp(a, "--blocksPerGrid")) g = atoi(v), i++;
            else if (!strcmp(a, "-b") || !strcmp(a, "--threadsPerBlock")) b = atoi(v), i++;
            else if (!strcmp(a, "--timeout-ms")) g_timeout_s = atof(v) / 1000.0, i++;
            else if (!strcmp(a, "--max-seconds")) max_seconds = atof(v), i++;
            else if (!strcmp(a, "-v") || !strcmp(a, "--verbose")) {
            } else if (a[0] == '-' && i + 1 < argc && argv[i + 1][0] != '-') i++;
        }
    }
    if (n == 0) n = (g ? g : 1) * (b ? b : 1);
    if (n < 1 || n > MAXR) {
        fprintf(stderr, "hostmpi: bad rank count %d\n", n);
        return 1;
    }
    const int prog_argc = pos >= 0 ? pos : argc;
    void* seg = mmap(nullptr, sizeof(Shm), PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
    void* pool = mmap(nullptr, POOL_BYTES, PROT_READ | PROT_WRITE,
                      MAP_SHARED | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (seg == MAP_FAILED || pool == MAP_FAILED) {
        perror("hostmpi: mmap");
        return 1;
    }
    g_shm = (Shm*)seg;
    memset(g_shm, 0, sizeof(Shm));
    g_shm->nranks = n;
    g_shm->pool = (char*)pool;
    g_shm->bump = 0;
    g_shm->end = POOL_BYTES;
    pthread_mutexattr_t ma;
    pthread_condattr_t ca;
    pthread_mutexattr_init(&ma);
    pthread_mutexattr_setpshared(&ma, PTHREAD_PROCESS_SHARED);
    pthread_condattr_init(&ca);
    pthread_condattr_setpshared(&ca, PTHREAD_PROCESS_SHARED);
    pthread_mutex_init(&g_shm->pool_mu, &ma);
    pthread_cond_init(&g_shm->pool_cv, &ca);
    for (int r = 0; r < n; r++) {
        pthread_mutex_init(&g_shm->box[r].mu, &ma);
        pthread_cond_init(&g_shm->box[r].cv, &ca);
    }
    fflush(stdout);
    fflush(stderr);
    std::vector<pid_t> pids(n);
    for (int r = 0; r < n; r++) {
        pid_t p = fork();
        if (p < 0) {
            perror("hostmpi: fork");
            g_shm->abort_flag = 1;
            return 1;
        }
        if (p == 0) {
            g_rank = r;
            g_size = n;
            std::vector<int> all(n);
            for (int i = 0; i < n; i++) all[i] = i;
            g_world_obj.ctx = 1;
            g_world_obj.size = n;
            g_world_obj.rank = r;
            g_world_obj.members = all;
            g_world_obj.topo_ndims = 0;
            g_self_obj.ctx = 2;
            g_self_obj.size = 1;
            g_self_obj.rank = 0;
            g_self_obj.members = std::vector<int>{r};
            g_self_obj.topo_ndims = 0;
            g_group_world_obj.members = all;
            g_group_world_obj.builtin = true;
            g_group_empty_obj.builtin = true;
            int rc = hostmpi_user_main(prog_argc, argv);
            fflush(stdout);
            fflush(stderr);
            _exit(rc & 0xff);
        }
        pids[r] = p;
    }
    int worst = 0, alive = n;
    const double t0 = now();
    double abort_since = -1;
    while (alive > 0) {
        int status = 0;
        pid_t p = waitpid(-1, &status, WNOHANG);
        if (p > 0) {
            alive--;
            int code = WIFEXITED(status) ? WEXITSTATUS(status) : 128 + WTERMSIG(status);
            if (code != 0) {
                worst = worst ? worst : code;
                g_shm->abort_flag = 1;
            }
            continue;
        }
        if (g_shm->abort_flag && abort_since < 0) abort_since = now();
        if ((abort_since >= 0 && now() - abort_since > 5.0) || now() - t0 > max_seconds) {
            if (now() - t0 > max_seconds) fprintf(stderr, "hostmpi: wall-clock limit exceeded\n");
            for (pid_t q : pids) kill(q, SIGKILL);
            worst = worst ? worst : 3;
            while (waitpid(-1, &status, 0) > 0) {
            }
            break;
        }
        usleep(500);
    }
    return worst ? 1 : 0;
}
