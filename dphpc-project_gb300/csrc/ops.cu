// Datatypes and reduction operators.
//
// Operator semantics and the (operator, type-class) legality table follow
// gpu_libs/gpu_mpi/operators.cu:73-200: MAX/MIN on integer and floating types,
// SUM/PROD also on complex types, LAND/LOR/LXOR on integer and logical types,
// BAND/BOR/BXOR on integer and byte types.  MAXLOC/MINLOC, which the reference
// declares but cannot instantiate, work here on the pair types.  Every
// operator is applied as inout = op(in, inout) (operators.cu:216-218) and the
// MAX/MIN tie rules are the reference's (`a > b ? a : b`, `a > b ? b : a`).
// Logical XOR uses MPI's definition (!a != !b); it equals the reference's
// `a != b` on 0/1 inputs.  Complex products use round-to-nearest intrinsics
// so that no multiply-add is contracted and results match a host fold bit
// for bit.
#include "rt.cuh"

#define GPUMPI_OP_OBJ_F(name, idx) {idx, 1, nullptr}
#define GPUMPI_OP_OBJ_SEP ,
__device__ MPI_Op_impl gm_builtin_ops[GPUMPI_NUM_BUILTIN_OPS] = {
    GPUMPI_OPS_LIST(GPUMPI_OP_OBJ_F, GPUMPI_OP_OBJ_SEP)};
#undef GPUMPI_OP_OBJ_F
#undef GPUMPI_OP_OBJ_SEP

#define GPUMPI_OP_DEF_F(name, idx) __device__ MPI_Op name = &gm_builtin_ops[idx];
#define GPUMPI_OP_DEF_SEP
GPUMPI_OPS_LIST(GPUMPI_OP_DEF_F, GPUMPI_OP_DEF_SEP)
#undef GPUMPI_OP_DEF_F
#undef GPUMPI_OP_DEF_SEP

namespace gm {

enum TypeClass { TC_INT, TC_FLOAT, TC_LOGICAL, TC_COMPLEX, TC_BYTE, TC_TEXT, TC_PAIR, TC_BAD };

// Canonical element kinds (one template instantiation per kind).
enum Canon {
    K_I8, K_U8, K_I16, K_U16, K_I32, K_U32, K_I64, K_U64, K_F32, K_F64, K_BOOL, K_CF32, K_CF64,
    K_2INT, K_FLOATINT, K_DOUBLEINT, K_LONGINT, K_OPAQUE1, K_OPAQUE4, K_BAD
};

struct TypeInfo {
    int size;
    int canon;
    int cls;
};

// Element kind and class of basic datatype t (the size field is filled by basic_info).
static __device__ TypeInfo basic_kind(int t) {
    switch (t) {
        case MPI_CHAR: return {1, K_OPAQUE1, TC_TEXT};
        case MPI_SHORT: return {2, K_I16, TC_INT};
        case MPI_INT: return {4, K_I32, TC_INT};
        case MPI_LONG: return {8, K_I64, TC_INT};
        case MPI_LONG_LONG_INT: return {8, K_I64, TC_INT};
        case MPI_LONG_LONG: return {8, K_I64, TC_INT};
        case MPI_SIGNED_CHAR: return {1, K_I8, TC_INT};
        case MPI_UNSIGNED_CHAR: return {1, K_U8, TC_INT};
        case MPI_UNSIGNED_SHORT: return {2, K_U16, TC_INT};
        case MPI_UNSIGNED: return {4, K_U32, TC_INT};
        case MPI_UNSIGNED_LONG: return {8, K_U64, TC_INT};
        case MPI_UNSIGNED_LONG_LONG: return {8, K_U64, TC_INT};
        case MPI_FLOAT: return {4, K_F32, TC_FLOAT};
        case MPI_DOUBLE: return {8, K_F64, TC_FLOAT};
        case MPI_LONG_DOUBLE: return {8, K_F64, TC_FLOAT};
        case MPI_WCHAR: return {4, K_OPAQUE4, TC_TEXT};
        case MPI_C_BOOL: return {1, K_BOOL, TC_LOGICAL};
        case MPI_INT8_T: return {1, K_I8, TC_INT};
        case MPI_INT16_T: return {2, K_I16, TC_INT};
        case MPI_INT32_T: return {4, K_I32, TC_INT};
        case MPI_INT64_T: return {8, K_I64, TC_INT};
        case MPI_UINT8_T: return {1, K_U8, TC_INT};
        case MPI_UINT16_T: return {2, K_U16, TC_INT};
        case MPI_UINT32_T: return {4, K_U32, TC_INT};
        case MPI_UINT64_T: return {8, K_U64, TC_INT};
        case MPI_C_COMPLEX: return {8, K_CF32, TC_COMPLEX};
        case MPI_C_FLOAT_COMPLEX: return {8, K_CF32, TC_COMPLEX};
        case MPI_C_DOUBLE_COMPLEX: return {16, K_CF64, TC_COMPLEX};
        case MPI_C_LONG_DOUBLE_COMPLEX: return {16, K_CF64, TC_COMPLEX};
        case MPI_BYTE: return {1, K_U8, TC_BYTE};
        case MPI_2INT: return {8, K_2INT, TC_PAIR};
        case MPI_FLOAT_INT: return {8, K_FLOATINT, TC_PAIR};
        case MPI_DOUBLE_INT: return {16, K_DOUBLEINT, TC_PAIR};
        case MPI_LONG_INT: return {16, K_LONGINT, TC_PAIR};
        case MPI_PACKED: return {1, K_OPAQUE1, TC_BYTE};
        default: return {-1, K_BAD, TC_BAD};
    }
}

// Size (from the datatype list's C types), element kind and class of basic datatype t.
static __device__ TypeInfo basic_info(int t) {
    TypeInfo ti = basic_kind(t);
    if (ti.canon != K_BAD) ti.size = basic_size(t);
    return ti;
}

__device__ int dtype_base(MPI_Datatype t, int* mult) {
    int ti = (int)t;
    if (ti >= 0 && ti < GPUMPI_NUM_BASIC_TYPES) {
        *mult = 1;
        return ti;
    }
    if (ti >= GPUMPI_FIRST_DERIVED_TYPE) {
        RankPriv* p = bctx().priv;
        int k = ti - GPUMPI_FIRST_DERIVED_TYPE;
        if (k < p->dt_used && p->dt_count[k] >= 0) {
            *mult = p->dt_count[k];
            return p->dt_base[k];
        }
    }
    *mult = 0;
    return -1;
}

__device__ int dtype_size(MPI_Datatype t) {
    int mult;
    int b = dtype_base(t, &mult);
    if (b < 0) return -1;
    return basic_info(b).size * mult;
}

static __device__ bool legal(int opi, int cls) {
    switch (opi) {
        case 0: case 1: return cls == TC_INT || cls == TC_FLOAT;
        case 2: case 3: return cls == TC_INT || cls == TC_FLOAT || cls == TC_COMPLEX;
        case 4: case 6: case 8: return cls == TC_INT || cls == TC_LOGICAL;
        case 5: case 7: case 9: return cls == TC_INT || cls == TC_BYTE;
        case 10: case 11: return cls == TC_PAIR;
        default: return false;
    }
}

// MPI_SUCCESS when `op` may reduce `t`, else MPI_ERR_OP.
__device__ int op_check(MPI_Op op, MPI_Datatype t) {
    if (op == nullptr) return MPI_ERR_OP;
    if (op->builtin < 0) return op->fn ? MPI_SUCCESS : MPI_ERR_OP;
    int mult;
    int b = dtype_base(t, &mult);
    if (b < 0) return MPI_ERR_TYPE;
    return legal(op->builtin, basic_info(b).cls) ? MPI_SUCCESS : MPI_ERR_OP;
}

// ---------------------------------------------------------------- operators
template <class T> struct OMax { __device__ static T f(T a, T b) { return a > b ? a : b; } };
template <class T> struct OMin { __device__ static T f(T a, T b) { return a > b ? b : a; } };
template <class T> struct OSum { __device__ static T f(T a, T b) { return (T)(a + b); } };
template <class T> struct OProd { __device__ static T f(T a, T b) { return (T)(a * b); } };
template <class T> struct OLAnd { __device__ static T f(T a, T b) { return (T)(a && b); } };
template <class T> struct OLOr { __device__ static T f(T a, T b) { return (T)(a || b); } };
template <class T> struct OLXor { __device__ static T f(T a, T b) { return (T)((!a) != (!b)); } };
template <class T> struct OBAnd { __device__ static T f(T a, T b) { return (T)(a & b); } };
template <class T> struct OBOr { __device__ static T f(T a, T b) { return (T)(a | b); } };
template <class T> struct OBXor { __device__ static T f(T a, T b) { return (T)(a ^ b); } };

template <> struct OSum<float> { __device__ static float f(float a, float b) { return __fadd_rn(a, b); } };
template <> struct OSum<double> { __device__ static double f(double a, double b) { return __dadd_rn(a, b); } };
template <> struct OProd<float> { __device__ static float f(float a, float b) { return __fmul_rn(a, b); } };
template <> struct OProd<double> { __device__ static double f(double a, double b) { return __dmul_rn(a, b); } };

template <> struct OSum<gpumpi_cfloat> {
    __device__ static gpumpi_cfloat f(gpumpi_cfloat a, gpumpi_cfloat b) {
        return {__fadd_rn(a.re, b.re), __fadd_rn(a.im, b.im)};
    }
};
template <> struct OSum<gpumpi_cdouble> {
    __device__ static gpumpi_cdouble f(gpumpi_cdouble a, gpumpi_cdouble b) {
        return {__dadd_rn(a.re, b.re), __dadd_rn(a.im, b.im)};
    }
};
template <> struct OProd<gpumpi_cfloat> {
    __device__ static gpumpi_cfloat f(gpumpi_cfloat a, gpumpi_cfloat b) {
        return {__fsub_rn(__fmul_rn(a.re, b.re), __fmul_rn(a.im, b.im)),
                __fadd_rn(__fmul_rn(a.re, b.im), __fmul_rn(a.im, b.re))};
    }
};
template <> struct OProd<gpumpi_cdouble> {
    __device__ static gpumpi_cdouble f(gpumpi_cdouble a, gpumpi_cdouble b) {
        return {__dsub_rn(__dmul_rn(a.re, b.re), __dmul_rn(a.im, b.im)),
                __dadd_rn(__dmul_rn(a.re, b.im), __dmul_rn(a.im, b.re))};
    }
};
template <class T> struct OMaxLoc {
    __device__ static T f(T a, T b) {
        if (a.val > b.val) return a;
        if (a.val < b.val) return b;
        return a.idx < b.idx ? a : b;
    }
};
template <class T> struct OMinLoc {
    __device__ static T f(T a, T b) {
        if (a.val > b.val) return b;
        if (a.val < b.val) return a;
        return a.idx < b.idx ? a : b;
    }
};

// ---------------------------------------------------------------- fold kernels
// Input q's base (+ in_off): from the block's pointer table in shared memory
// when fold_range built one, else from the communicator's published table.
template <class T>
static __device__ __forceinline__ const T* in_ptr(const Pub* pub, int q, u64 in_off, const char* const* ptab) {
    if (ptab) return reinterpret_cast<const T*>(ptab[q]);
    return reinterpret_cast<const T*>((const char*)ldcg(&pub[q].sbuf) + in_off);
}

// Scalar path: any element type, any alignment.
template <class T, class O>
static __device__ void fold_scalar(T* out, const Pub* pub, int nin, u64 in_off, u64 lo, u64 hi,
                                   int tid, int T_, const char* const* ptab) {
    for (u64 i = lo + tid; i < hi; i += T_) {
        T acc = ldcg(in_ptr<T>(pub, 0, in_off, ptab) + i);
        for (int q = 1; q < nin; q++) acc = O::f(ldcg(in_ptr<T>(pub, q, in_off, ptab) + i), acc);
        out[i - lo] = acc;
    }
}

template <class T, class O>
static __device__ __forceinline__ void combine(uint4& acc, const uint4& x) {
    constexpr int V = 16 / sizeof(T);
    T* a = reinterpret_cast<T*>(&acc);
    const T* xe = reinterpret_cast<const T*>(&x);
#pragma unroll
    for (int e = 0; e < V; e++) a[e] = O::f(xe[e], a[e]);
}

// 16-byte vector path for 4- and 8-byte element types when every input and
// the output are 16-byte aligned at element lo.
// With a pointer table in shared memory: one vector per thread at a time and
// QU input ranks' vectors in flight, folded in rank order.
// Without one: four independent vectors per thread, each input's base loaded
// from the communicator's table.
template <class T, class O>
static __device__ void fold_vec(T* out, const Pub* pub, int nin, u64 in_off, u64 lo, u64 hi,
                                int tid, int T_, const char* const* ptab) {
    constexpr int V = 16 / sizeof(T);
    const u64 n = hi - lo;
    const u64 nvec = n / V;
    uint4* ov = reinterpret_cast<uint4*>(out);
    u64 v = tid;
    if (ptab) {
        constexpr int QU = 8;
        for (; v < nvec; v += T_) {
            uint4 acc = __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[0]) + lo) + v);
            int q = 1;
            for (; q + QU <= nin; q += QU) {
                uint4 x[QU];
#pragma unroll
                for (int k = 0; k < QU; k++)
                    x[k] = __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[q + k]) + lo) + v);
#pragma unroll
                for (int k = 0; k < QU; k++) combine<T, O>(acc, x[k]);
            }
            for (; q < nin; q++)
                combine<T, O>(acc, __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[q]) + lo) + v));
            ov[v] = acc;
        }
    } else {
        constexpr int U = 4;
        for (; v + (U - 1) * (u64)T_ < nvec; v += (u64)U * T_) {
            uint4 acc[U];
            const uint4* b0 = reinterpret_cast<const uint4*>(in_ptr<T>(pub, 0, in_off, ptab) + lo);
#pragma unroll
            for (int k = 0; k < U; k++) acc[k] = __ldcg(b0 + v + (u64)k * T_);
            for (int q = 1; q < nin; q++) {
                const uint4* bq = reinterpret_cast<const uint4*>(in_ptr<T>(pub, q, in_off, ptab) + lo);
                uint4 x[U];
#pragma unroll
                for (int k = 0; k < U; k++) x[k] = __ldcg(bq + v + (u64)k * T_);
#pragma unroll
                for (int k = 0; k < U; k++) combine<T, O>(acc[k], x[k]);
            }
#pragma unroll
            for (int k = 0; k < U; k++) ov[v + (u64)k * T_] = acc[k];
        }
        for (; v < nvec; v += T_) {
            uint4 acc = __ldcg(reinterpret_cast<const uint4*>(in_ptr<T>(pub, 0, in_off, ptab) + lo) + v);
            for (int q = 1; q < nin; q++)
                combine<T, O>(acc, __ldcg(reinterpret_cast<const uint4*>(in_ptr<T>(pub, q, in_off, ptab) + lo) + v));
            ov[v] = acc;
        }
    }
    const u64 done = nvec * V;
    if (done < n) fold_scalar<T, O>(out + done, pub, nin, in_off, lo + done, hi, tid, T_, ptab);
}

// Fold [lo, hi) of every input and write the result at the same place in
// every output (ptab: inputs, otab: outputs, both in shared memory and 16-byte
// aligned).  QU input ranks' vectors in flight per thread, folded in rank order.
template <class T, class O>
static __device__ __noinline__ void fold_push_t(const char* const* ptab, const char* const* otab, int nin, u64 lo,
                                                u64 hi, int tid, int T_) {
    constexpr int V = 16 / sizeof(T);
    constexpr int QU = 8;
    const u64 n = hi - lo;
    const u64 nvec = n / V;
    for (u64 v = tid; v < nvec; v += T_) {
        uint4 acc = __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[0]) + lo) + v);
        int q = 1;
        for (; q + QU <= nin; q += QU) {
            uint4 x[QU];
#pragma unroll
            for (int k = 0; k < QU; k++)
                x[k] = __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[q + k]) + lo) + v);
#pragma unroll
            for (int k = 0; k < QU; k++) combine<T, O>(acc, x[k]);
        }
        for (; q < nin; q++)
            combine<T, O>(acc, __ldcg(reinterpret_cast<const uint4*>(reinterpret_cast<const T*>(ptab[q]) + lo) + v));
        for (int r = 0; r < nin; r++)
            reinterpret_cast<uint4*>(const_cast<T*>(reinterpret_cast<const T*>(otab[r]) + lo))[v] = acc;
    }
    for (u64 i = lo + nvec * V + tid; i < hi; i += T_) {
        T acc = ldcg(reinterpret_cast<const T*>(ptab[0]) + i);
        for (int q = 1; q < nin; q++) acc = O::f(ldcg(reinterpret_cast<const T*>(ptab[q]) + i), acc);
        for (int r = 0; r < nin; r++) const_cast<T*>(reinterpret_cast<const T*>(otab[r]))[i] = acc;
    }
}

// Gather path for short folds (few elements, many inputs): the block first
// loads all nin * m input elements into shared memory, 8 independent loads in
// flight per thread, then thread i folds element i in rank order from there.
// A thread-per-element fold would instead wait one memory round trip per
// input (256 of them for a 256-rank communicator).  `g` is the gather area
// (nin * m elements of T, shared memory).
template <class T, class O>
static __device__ void fold_gather(T* out, const Pub* pub, int nin, u64 in_off, u64 lo, u64 hi, int tid,
                                   int T_, const char* const* ptab, T* g) {
    const u64 m = hi - lo;
    const u64 total = m * (u64)nin;
    constexpr int U = 8;
    for (u64 k0 = (u64)tid; k0 < total; k0 += (u64)U * T_) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const u64 k = k0 + (u64)u * T_;
            if (k < total) v[u] = ldcg(in_ptr<T>(pub, (int)(k / m), in_off, ptab) + lo + k % m);
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const u64 k = k0 + (u64)u * T_;
            if (k < total) g[k] = v[u];
        }
    }
    bsync();
    for (u64 i = tid; i < m; i += T_) {
        T acc = g[i];
        for (int q = 1; q < nin; q++) acc = O::f(g[(u64)q * m + i], acc);
        out[i] = acc;
    }
}

// Shared memory available to fold_gather after the pointer table (bytes), and its start.
static __device__ __forceinline__ u32 gather_bytes(int nin, char** at) {
    extern __shared__ __align__(16) char gm_dsmem[];
    const u32 tab = ((u32)nin * (u32)sizeof(char*) + 15u) & ~15u;
    const u32 avail = bulk_stage_bytes();
    *at = gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES + tab;
    return avail > tab ? avail - tab : 0;
}

// One out-of-line function per (type, operator): each gets its own register
// allocation instead of sharing one across the whole dispatch switch.
template <class T, class O>
static __device__ __noinline__ void fold_t(void* outv, const Pub* pub, int nin, u64 in_off, u64 lo, u64 hi,
                                           int tid, int T_, const char* const* ptab) {
    T* out = reinterpret_cast<T*>(outv);
    if (nin >= 8 && hi - lo <= 4 * (u64)T_) {
        char* at = nullptr;
        if ((hi - lo) * (u64)nin * sizeof(T) <= gather_bytes(nin, &at) && alignof(T) <= 16) {
            fold_gather<T, O>(out, pub, nin, in_off, lo, hi, tid, T_, ptab, reinterpret_cast<T*>(at));
            return;
        }
    }
    if constexpr (sizeof(T) == 4 || sizeof(T) == 8) {
        bool aligned = ((uintptr_t)out & 15) == 0;
        for (int q = 0; q < nin && aligned; q++)
            aligned = (((uintptr_t)(in_ptr<T>(pub, q, in_off, ptab) + lo)) & 15) == 0;
        if (aligned) {
            fold_vec<T, O>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            return;
        }
    }
    fold_scalar<T, O>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
}

template <template <class> class O>
static __device__ void fold_numeric(int canon, void* out, const Pub* pub, int nin, u64 in_off,
                                    u64 lo, u64 hi, int tid, int T_, const char* const* ptab) {
    switch (canon) {
        case K_I8: fold_t<signed char, O<signed char>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_U8: fold_t<unsigned char, O<unsigned char>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_I16: fold_t<short, O<short>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_U16: fold_t<unsigned short, O<unsigned short>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_I32: fold_t<int, O<int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_U32: fold_t<unsigned, O<unsigned>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_I64: fold_t<long long, O<long long>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case K_U64: fold_t<unsigned long long, O<unsigned long long>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        default: break;
    }
}

template <template <class> class O>
static __device__ void fold_float(int canon, void* out, const Pub* pub, int nin, u64 in_off,
                                  u64 lo, u64 hi, int tid, int T_, const char* const* ptab) {
    if (canon == K_F32) fold_t<float, O<float>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
    else if (canon == K_F64) fold_t<double, O<double>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
}

static __device__ void fold_user(MPI_User_function* fn, MPI_Datatype dt, int es, void* out,
                                 const Pub* pub, int nin, u64 in_off, u64 lo, u64 hi, int tid,
                                 int T_) {
    // Contiguous chunks per thread; each chunk folds in rank order.
    const u64 n = hi - lo;
    const u64 per = (n + T_ - 1) / T_;
    const u64 c0 = (u64)tid * per;
    if (c0 >= n) return;
    u64 c1 = c0 + per;
    if (c1 > n) c1 = n;
    char* o = (char*)out + c0 * es;
    const char* i0 = (const char*)ldcg(&pub[0].sbuf) + in_off + (lo + c0) * es;
    for (u64 k = 0; k < (c1 - c0) * es; k++) o[k] = __ldcg(i0 + k);
    int len = (int)(c1 - c0);
    MPI_Datatype d = dt;
    for (int q = 1; q < nin; q++) {
        const char* iq = (const char*)ldcg(&pub[q].sbuf) + in_off + (lo + c0) * es;
        fn((void*)iq, o, &len, &d);
    }
}

// ---------------------------------------------------------------- bulk-staged push
// The same fold with the inputs staged through shared memory: cp.async.bulk
// loads one chunk of 16*T bytes (one vector per thread) of one input into a
// ring of ns stages, each with a "full" mbarrier (completed by the load's
// bytes) and an "empty" mbarrier (one arrival per thread once it has read its
// vector).  Loads are issued in fold order (chunk by chunk, input rank by
// input rank) by thread 0, which refills a stage one step after consuming it,
// so up to ns - 1 loads are in flight whatever the registers allow.  Results
// go to the outputs with ordinary stores once a chunk's last input is folded.
// Every wait is bounded by the job's timeout; returns 0 or an error code.
// 0 once the phase of `parity` has completed; 1 once the job has failed, 2
// after the job's timeout.
static __device__ __forceinline__ int mbar_wait(u32 bar, u32 parity, u64 t0, const Job* j) {
    for (unsigned it = 0;; it++) {
        u32 done = 0;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return 0;
        if ((it & 15u) == 15u) {
            if (ld_relaxed_int(&j->status[0]) != 0) return 1;
            if (gtime() - t0 > j->timeout_ns) return 2;
        }
    }
}

// Thread 0: load chunk ic of input iq (nv vectors from element lo) into stage ist.
static __device__ __forceinline__ void fold_bulk_issue(const char* src, u32 len, u32 dst_s, u32 full) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full), "r"(len) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst_s), "l"(src), "r"(len), "r"(full) : "memory");
}

template <class T, class O>
static __device__ __noinline__ int fold_push_bulk_t(const char* const* ptab, const char* const* otab, int nin, u64 lo,
                                                    u64 nvec, int tid, int T_, char* ring, u64* bars, int ns) {
    // vectors per stage: one per thread, or every vector of a short segment
    const u32 VPS = nvec < (u64)T_ ? (u32)nvec : (u32)T_;
    const u32 C = VPS * 16;
    const u64 K = (nvec + VPS - 1) / VPS * (u64)nin;
    const u64 off = lo * sizeof(T);
    const u32 ring_s = (u32)__cvta_generic_to_shared(ring);
    const u32 full_s = (u32)__cvta_generic_to_shared(bars);   // full[0..ns), then empty[0..ns)
    const u32 empty_s = full_s + 8u * (u32)ns;
    Job* j = bctx().job;
    // issue side (thread 0): the next load's step, first vector, input rank and stage
    u64 issued = 0, iv0 = 0;
    int iq = 0, ist = 0;
#define GM_FOLD_ISSUE()                                                                                \
    do {                                                                                               \
        const u64 nv_ = nvec - iv0 < (u64)VPS ? nvec - iv0 : (u64)VPS;                                 \
        fold_bulk_issue(ptab[iq] + off + iv0 * 16, (u32)(nv_ * 16), ring_s + (u32)ist * C,             \
                        full_s + 8u * (u32)ist);                                                       \
        issued++;                                                                                      \
        if (++iq == nin) {                                                                             \
            iq = 0;                                                                                    \
            iv0 += (u64)VPS;                                                                           \
        }                                                                                              \
        if (++ist == ns) ist = 0;                                                                      \
    } while (0)
    if (tid == 0)
        while (issued < K && issued < (u64)ns) GM_FOLD_ISSUE();
    int err = 0;
    uint4 acc = make_uint4(0, 0, 0, 0);
    const u64 t0 = gtime();
    // consume side (every thread): this thread's vector, input rank, stage and phase
    u64 v = (u64)tid;
    int q = 0, st = 0, pst = ns - 1;
    u32 par = 0, ppar = 1;
    for (u64 k = 0; k < K; k++) {
        err = mbar_wait(full_s + 8u * (u32)st, par, t0, j);
        if (err) break;
        if (v < nvec) {
            const uint4 x = reinterpret_cast<const uint4*>(ring + st * C)[tid];
            if (q == 0) acc = x;
            else combine<T, O>(acc, x);
        }
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(empty_s + 8u * (u32)st) : "memory");
        if (tid == 0 && k >= 1 && issued < K) {
            // refill the stage of step k - 1 once every thread has read it
            err = mbar_wait(empty_s + 8u * (u32)pst, ppar, t0, j);
            if (err) break;
            GM_FOLD_ISSUE();
        }
        pst = st;
        ppar = par;
        if (++st == ns) {
            st = 0;
            par ^= 1u;
        }
        if (++q == nin) {
            if (v < nvec)
                for (int r = 0; r < nin; r++) reinterpret_cast<uint4*>(const_cast<char*>(otab[r]) + off)[v] = acc;
            q = 0;
            v += (u64)VPS;
        }
    }
#undef GM_FOLD_ISSUE
    if (tid == 0 && err) {
        // the loads still in flight write the ring: wait for them (bounded) before
        // the block leaves; the caller keeps the block off the staging area
        const u64 t1 = gtime();
        const u64 first = issued > (u64)ns ? issued - (u64)ns : 0;
        for (u64 k = first; k < issued; k++) {
            const u32 bar = full_s + 8u * (u32)(k % (u64)ns);
            const u32 p2 = (u32)((k / (u64)ns) & 1);
            u32 done = 0;
            while (!done && gtime() - t1 < j->timeout_ns)
                asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                             : "=r"(done) : "r"(bar), "r"(p2) : "memory");
        }
    }
    if (err == 2) job_fail(j, bctx().rank, GPUMPI_ERR_TIMEOUT, "bulk fold did not complete");
    return err ? fail_code(j) : 0;
}

template <template <class> class O>
static __device__ int fold_push_bulk_op(int canon, const char* const* ptab, const char* const* otab, int nin, u64 lo,
                                        u64 nvec, int tid, int T_, char* ring, u64* bars, int ns) {
    switch (canon) {
        case K_I32: return fold_push_bulk_t<int, O<int>>(ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns);
        case K_U32: return fold_push_bulk_t<unsigned, O<unsigned>>(ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns);
        case K_I64: return fold_push_bulk_t<long long, O<long long>>(ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns);
        case K_U64:
            return fold_push_bulk_t<unsigned long long, O<unsigned long long>>(ptab, otab, nin, lo, nvec, tid, T_, ring,
                                                                               bars, ns);
        case K_F32: return fold_push_bulk_t<float, O<float>>(ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns);
        default: return fold_push_bulk_t<double, O<double>>(ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns);
    }
}

template <template <class> class O>
static __device__ bool fold_push_op(int canon, const char* const* ptab, const char* const* otab, int nin, u64 lo,
                                    u64 hi, int tid, int T_) {
    switch (canon) {
        case K_I32: fold_push_t<int, O<int>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        case K_U32: fold_push_t<unsigned, O<unsigned>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        case K_I64: fold_push_t<long long, O<long long>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        case K_U64: fold_push_t<unsigned long long, O<unsigned long long>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        case K_F32: fold_push_t<float, O<float>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        case K_F64: fold_push_t<double, O<double>>(ptab, otab, nin, lo, hi, tid, T_); return true;
        default: return false;
    }
}

static __device__ __forceinline__ bool push_type(int canon) {
    return canon == K_I32 || canon == K_U32 || canon == K_I64 || canon == K_U64 || canon == K_F32 || canon == K_F64;
}

// Allreduce, pushing form: this rank folds [lo, hi) of every rank's input in
// rank order and stores the result into every rank's receive buffer.  Returns
// false (the same on every rank and every thread, since it depends only on the
// launch, the operator and the published buffers) when the form does not
// apply: no staging area for the two pointer tables, a user or bitwise
// operator, a type that is not 4 or 8 bytes, or a buffer not 16-byte aligned.
__device__ bool fold_range_push(int opi, MPI_Datatype base, const Pub* pub, int nin, u64 lo, u64 hi, int tid,
                                int T_) {
    if (opi < 0 || opi > 3 || nin < 2) return false;
    const int canon = basic_info((int)base).canon;
    if (!push_type(canon) || bulk_stage_bytes() < (u32)(2 * nin * sizeof(char*))) return false;
    extern __shared__ __align__(16) char gm_dsmem[];
    const char** ptab = reinterpret_cast<const char**>(gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES);
    const char** otab = ptab + nin;
    int bad = 0;
    for (int q = tid; q < nin; q += T_) {
        ptab[q] = (const char*)ldcg(&pub[q].sbuf);
        otab[q] = (const char*)ldcg(&pub[q].rbuf);
        bad |= ((((uintptr_t)ptab[q]) | ((uintptr_t)otab[q])) & 15) != 0;
    }
    if (bar_or(bad, T_)) return false;
    // bulk staging: the ring and its 2 * ns mbarriers after the two tables
    const u64 esz = basic_info((int)base).size;
    const u64 nvec = hi > lo ? (hi - lo) * esz / 16 : 0;
    const u32 tab_bytes = (u32)(2 * nin * sizeof(char*));
    const u32 C = (nvec < (u64)T_ ? (u32)nvec : (u32)T_) * 16;   // a stage: one vector per thread at most
    const u32 avail = bulk_stage_bytes();
    int ns = 0;
    if (!bctx().bulk_broken && nvec >= 16 && avail > tab_bytes + 256) {
        ns = (int)((avail - tab_bytes - 256) / C);
        if (ns > 16) ns = 16;
    }
    if (ns >= 4) {
        u64* bars = reinterpret_cast<u64*>(gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES + ((tab_bytes + 15) & ~15u));
        char* ring = reinterpret_cast<char*>(bars) + 256;
        if (tid < 2 * ns)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"((u32)__cvta_generic_to_shared(&bars[tid])),
                         "r"(tid < ns ? 1 : T_) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("fence.proxy.async.global;" ::: "memory");
        bsync();
        int rc = 0;
        switch (opi) {
            case 0: rc = fold_push_bulk_op<OMax>(canon, ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns); break;
            case 1: rc = fold_push_bulk_op<OMin>(canon, ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns); break;
            case 2: rc = fold_push_bulk_op<OSum>(canon, ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns); break;
            default: rc = fold_push_bulk_op<OProd>(canon, ptab, otab, nin, lo, nvec, tid, T_, ring, bars, ns); break;
        }
        if (bar_or(rc != 0, T_)) {
            bctx().bulk_broken = 1;   // loads may still be in flight into the ring
            return true;              // the job has failed; peers leave their waits
        }
        if (tid < 2 * ns)
            asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"((u32)__cvta_generic_to_shared(&bars[tid])) : "memory");
        // the elements after the last whole vector
        const u64 done = nvec * 16 / esz;
        if (lo + done < hi) {
            switch (opi) {
                case 0: fold_push_op<OMax>(canon, ptab, otab, nin, lo + done, hi, tid, T_); break;
                case 1: fold_push_op<OMin>(canon, ptab, otab, nin, lo + done, hi, tid, T_); break;
                case 2: fold_push_op<OSum>(canon, ptab, otab, nin, lo + done, hi, tid, T_); break;
                default: fold_push_op<OProd>(canon, ptab, otab, nin, lo + done, hi, tid, T_); break;
            }
        }
        bsync();
        return true;
    }
    if (hi > lo) {
        switch (opi) {
            case 0: fold_push_op<OMax>(canon, ptab, otab, nin, lo, hi, tid, T_); break;
            case 1: fold_push_op<OMin>(canon, ptab, otab, nin, lo, hi, tid, T_); break;
            case 2: fold_push_op<OSum>(canon, ptab, otab, nin, lo, hi, tid, T_); break;
            default: fold_push_op<OProd>(canon, ptab, otab, nin, lo, hi, tid, T_); break;
        }
    }
    bsync();
    return true;
}

__device__ void fold_range(int opi, MPI_User_function* ufn, MPI_Datatype base, int esize, void* out, const Pub* pub, int nin,
                           u64 in_off, u64 lo, u64 hi, int tid, int T_) {
    if (hi <= lo || nin <= 0) {
        bsync();
        return;
    }
    if (opi < 0) {
        fold_user(ufn, base, esize, out, pub, nin, in_off, lo, hi, tid, T_);
        bsync();
        return;
    }
    const int canon = basic_info((int)base).canon;
    // Input pointers (+ in_off) in the staging area of shared memory, when the
    // launch gave one: the fold then reads each input's base without a load
    // through L2.
    const char** ptab = nullptr;
    if (nin >= 2 && bulk_stage_bytes() >= (u32)nin * sizeof(char*)) {
        extern __shared__ __align__(16) char gm_dsmem[];
        ptab = reinterpret_cast<const char**>(gm_dsmem + BCTX_BYTES + BULK_BAR_BYTES);
        for (int q = tid; q < nin; q += T_) ptab[q] = (const char*)ldcg(&pub[q].sbuf) + in_off;
        bsync();
    }
    switch (opi) {
        case 0:
            fold_numeric<OMax>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            fold_float<OMax>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 1:
            fold_numeric<OMin>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            fold_float<OMin>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 2:
            fold_numeric<OSum>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            fold_float<OSum>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_CF32) fold_t<gpumpi_cfloat, OSum<gpumpi_cfloat>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_CF64) fold_t<gpumpi_cdouble, OSum<gpumpi_cdouble>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 3:
            fold_numeric<OProd>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            fold_float<OProd>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_CF32) fold_t<gpumpi_cfloat, OProd<gpumpi_cfloat>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_CF64) fold_t<gpumpi_cdouble, OProd<gpumpi_cdouble>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 4:
            fold_numeric<OLAnd>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_BOOL) fold_t<bool, OLAnd<bool>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 5: fold_numeric<OBAnd>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case 6:
            fold_numeric<OLOr>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_BOOL) fold_t<bool, OLOr<bool>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 7: fold_numeric<OBOr>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case 8:
            fold_numeric<OLXor>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            if (canon == K_BOOL) fold_t<bool, OLXor<bool>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            break;
        case 9: fold_numeric<OBXor>(canon, out, pub, nin, in_off, lo, hi, tid, T_, ptab); break;
        case 10:
        case 11: {
            const bool mx = opi == 10;
            if (canon == K_2INT) {
                if (mx) fold_t<gpumpi_2int, OMaxLoc<gpumpi_2int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
                else fold_t<gpumpi_2int, OMinLoc<gpumpi_2int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            } else if (canon == K_FLOATINT) {
                if (mx) fold_t<gpumpi_float_int, OMaxLoc<gpumpi_float_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
                else fold_t<gpumpi_float_int, OMinLoc<gpumpi_float_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            } else if (canon == K_DOUBLEINT) {
                if (mx) fold_t<gpumpi_double_int, OMaxLoc<gpumpi_double_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
                else fold_t<gpumpi_double_int, OMinLoc<gpumpi_double_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            } else if (canon == K_LONGINT) {
                if (mx) fold_t<gpumpi_long_int, OMaxLoc<gpumpi_long_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
                else fold_t<gpumpi_long_int, OMinLoc<gpumpi_long_int>>(out, pub, nin, in_off, lo, hi, tid, T_, ptab);
            }
            break;
        }
        default: break;
    }
    bsync();
}

}  // namespace gm
