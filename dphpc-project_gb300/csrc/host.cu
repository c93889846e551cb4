// Host side of the program launcher: option parsing compatible with the
// reference's "---gpumpi" syntax (gpu_libs/gpu_main/main.cu:49-98), job memory
// layout in HBM, co-residency check (main.cu:189-209, done here with the
// cooperative-launch occupancy query), launch, output drain and exit status.
#include <cuda_runtime.h>
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <time.h>

#include <string>
#include <atomic>
#include <map>
#include <mutex>
#include <vector>

#include "gpumpi.h"
#include "hostjob.h"

#include <map>
#include <mutex>
#include "rt.cuh"

static_assert(GPUMPI_DT_INT == MPI_INT && GPUMPI_DT_DOUBLE == MPI_DOUBLE && GPUMPI_DT_BYTE == MPI_BYTE &&
                  GPUMPI_DT_INT64 == MPI_INT64_T && GPUMPI_DT_FLOAT == MPI_FLOAT,
              "host datatype codes follow the device enum");

extern "C" size_t gpumpi_heap_meta_bytes();

namespace gm {

static char g_last_error[512] = "";

void set_last_error(const char* msg) {
    snprintf(g_last_error, sizeof(g_last_error), "%s", msg);
}

#define HCHECK(call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            char m_[400];                                                             \
            snprintf(m_, sizeof(m_), "%s failed: %s", #call, cudaGetErrorString(e_)); \
            set_last_error(m_);                                                       \
            fprintf(stderr, "GPUMPI: %s\n", m_);                                      \
            return GPUMPI_ECUDA;                                                      \
        }                                                                             \
    } while (0)

// ------------------------------------------------------------------ layout
struct Carver {
    size_t off = 0;
    size_t take(size_t bytes, size_t align = 256) {
        off = (off + align - 1) & ~(align - 1);
        size_t o = off;
        off += bytes;
        return o;
    }
};

void opts_defaults(gpumpi_opts* o) {
    if (o->stack_bytes == 0) o->stack_bytes = 16 * 1024;
    if (o->heap_bytes == 0) o->heap_bytes = (size_t)1 << 30;
    if (o->max_requests == 0) o->max_requests = 1024;
    if (o->eager_bytes == 0) o->eager_bytes = 4096;
    if (o->timeout_s <= 0) o->timeout_s = 60.0;
    if (o->out_bytes == 0) o->out_bytes = (size_t)16 << 20;
}

size_t job_footprint(const gpumpi_opts& o, int n) {
    HostJob tmp;
    return host_job_layout(tmp, o, n, 0, nullptr);
}

// Compute (and, when base != nullptr, fill) the layout of one job.
size_t host_job_layout(HostJob& hj, const gpumpi_opts& o, int n, int job_id, char* base) {
    Carver c;
    const size_t eager = (o.eager_bytes + 15) & ~(size_t)15;
    const u32 npages = (u32)((o.heap_bytes + 65535) / 65536);
    const size_t meta_bytes = gpumpi_heap_meta_bytes();
    // zeroed control region first
    size_t z0 = c.take(0);
    size_t o_mbox = c.take(sizeof(Mailbox) * (size_t)n, 128);
    size_t o_wcs = c.take(sizeof(CommShared), 128);
    size_t o_wpub = c.take(sizeof(Pub) * (size_t)n);
    size_t o_warr = c.take(sizeof(u64) * (size_t)n * 3);
    size_t o_scs = c.take(sizeof(CommShared) * (size_t)n, 128);
    size_t o_spub = c.take(sizeof(Pub) * (size_t)n);
    size_t o_sarr = c.take(sizeof(u64) * (size_t)n * 3);
    size_t o_status = c.take(sizeof(int) * 16);
    size_t o_ret = c.take(sizeof(int) * (size_t)n);
    size_t o_cldone = c.take(sizeof(u64) * (size_t)n);
    size_t o_offs = c.take(sizeof(u64) * 4);
    size_t o_hctl = c.take(heap_ctl_bytes());
    size_t o_meta = c.take(meta_bytes * npages);
    size_t o_arena = c.take(((size_t)4 << 20) + (size_t)n * 4096);
    size_t arena_bytes = ((size_t)4 << 20) + (size_t)n * 4096;
    size_t z1 = c.take(0);
    // not zeroed
    size_t o_clsp = c.take(sizeof(u32) * 12 * (size_t)npages);
    size_t o_eager = c.take(eager * MB_SLOTS * (size_t)n);
    size_t o_priv = c.take(sizeof(RankPriv) * (size_t)n);
    size_t o_req = c.take(sizeof(MPI_Request_impl) * (size_t)n * o.max_requests);
    size_t o_stage = c.take((size_t)STAGE_BYTES * n);
    size_t o_cscr = c.take((size_t)COLL_SCRATCH_BYTES * n);
    size_t o_out = c.take(o.out_bytes);
    size_t o_err = c.take(o.out_bytes);
    size_t o_errmsg = c.take(256);
    size_t o_heap = c.take((size_t)npages * 65536, 65536);
    size_t o_job = c.take(sizeof(Job));
    size_t total = c.take(0);
    hj.zero_off = z0;
    hj.zero_bytes = z1 - z0;
    hj.clsp_off = o_clsp;
    hj.clsp_bytes = sizeof(u32) * 12 * (size_t)npages;
    hj.total = total;
    hj.nranks = n;
    hj.job_off = o_job;
    if (!base) return total;
    hj.base = base;
    Job& j = hj.job;
    memset(&j, 0, sizeof(j));
    j.id = job_id;
    j.nranks = n;
    j.threads = o.threads_per_rank;
    j.max_requests = o.max_requests;
    j.timeout_ns = (u64)(o.timeout_s * 1e9);
    j.eager_bytes = eager;
    j.mbox = (Mailbox*)(base + o_mbox);
    j.eager = base + o_eager;
    j.priv = (RankPriv*)(base + o_priv);
    j.reqpool = (MPI_Request_impl*)(base + o_req);
    j.stage = base + o_stage;
    j.coll_scratch = base + o_cscr;
    j.world_cs = (CommShared*)(base + o_wcs);
    j.self_cs = (CommShared*)(base + o_scs);
    j.arena = base + o_arena;
    j.arena_bytes = arena_bytes;
    u64* offs = (u64*)(base + o_offs);
    j.out_off = offs + 0;
    j.errout_off = offs + 1;
    j.arena_off = offs + 2;
    j.out = base + o_out;
    j.errout = base + o_err;
    j.out_bytes = o.out_bytes;
    j.status = (int*)(base + o_status);
    j.retvals = (int*)(base + o_ret);
    j.cl_done = (u64*)(base + o_cldone);
    j.err_msg = base + o_errmsg;
    // heap
    Heap& h = j.heap;
    h.base = base + o_heap;
    h.bytes = (u64)npages * 65536;
    h.npages = npages;
    h.meta = (PageMeta*)(base + o_meta);
    heap_set_ctl(h, base + o_hctl);
    h.cls_pages = (u32*)(base + o_clsp);
    // communicator tables (host copies, uploaded by the caller)
    hj.world.size = n;
    hj.world.ctx = 1;
    hj.world.members = nullptr;
    hj.world.pub = (Pub*)(base + o_wpub);
    hj.world.arrive = (u64*)(base + o_warr);
    hj.world.mid = hj.world.arrive + n;
    hj.world.depart = hj.world.arrive + 2 * (size_t)n;
    hj.selfs.resize(n);
    for (int r = 0; r < n; r++) {
        CommShared& s = hj.selfs[r];
        memset(&s, 0, sizeof(s));
        s.size = 1;
        s.ctx = 2;
        s.self_member = r;
        s.members = (int*)(base + o_scs + sizeof(CommShared) * (size_t)r + offsetof(CommShared, self_member));
        s.pub = (Pub*)(base + o_spub) + r;
        s.arrive = (u64*)(base + o_sarr) + 3 * (size_t)r;
        s.mid = s.arrive + 1;
        s.depart = s.arrive + 2;
    }
    return total;
}

// Zero the control state and upload the job description.
int host_job_init(HostJob& hj, cudaStream_t st) {
    HCHECK(cudaMemsetAsync(hj.base + hj.zero_off, 0, hj.zero_bytes, st));
    HCHECK(cudaMemsetAsync(hj.base + hj.clsp_off, 0xff, hj.clsp_bytes, st));
    HCHECK(cudaMemcpyAsync(hj.job.world_cs, &hj.world, sizeof(CommShared), cudaMemcpyHostToDevice, st));
    HCHECK(cudaMemcpyAsync(hj.job.self_cs, hj.selfs.data(), sizeof(CommShared) * hj.selfs.size(),
                           cudaMemcpyHostToDevice, st));
    HCHECK(cudaMemcpyAsync(hj.base + hj.job_off, &hj.job, sizeof(Job), cudaMemcpyHostToDevice, st));
    return GPUMPI_OK;
}

// ------------------------------------------------------------------ args
static bool parse_size(const char* s, size_t* out) {
    char* e = nullptr;
    double v = strtod(s, &e);
    if (e == s || v < 0) return false;
    if (*e == 'k' || *e == 'K') v *= 1024.0;
    else if (*e == 'm' || *e == 'M') v *= 1024.0 * 1024.0;
    else if (*e == 'g' || *e == 'G') v *= 1024.0 * 1024.0 * 1024.0;
    *out = (size_t)v;
    return true;
}

}  // namespace gm

using namespace gm;

extern "C" const char* gpumpi_last_error(void) { return g_last_error; }

extern "C" int gpumpi_parse_args(int argc, char** argv, gpumpi_opts* o) {
    memset(o, 0, sizeof(*o));
    int pos = -1;
    for (int i = 0; i < argc; i++)
        if (strcmp(argv[i], "---gpumpi") == 0) pos = i;
    if (pos < 0) return -1;
    unsigned blocks = 0, threads = 0;
    for (int i = pos + 1; i < argc; i++) {
        std::string a = argv[i];
        std::string val;
        bool has_val = false;
        size_t eq = a.find('=');
        if (a.rfind("--", 0) == 0 && eq != std::string::npos) {
            val = a.substr(eq + 1);
            a = a.substr(0, eq);
            has_val = true;
        }
        auto next = [&](std::string* v) -> bool {
            if (has_val) {
                *v = val;
                return true;
            }
            if (i + 1 >= argc) return false;
            *v = argv[++i];
            return true;
        };
        std::string v;
        if (a == "-h" || a == "--help") {
            printf(
                "GPU MPI (GB300) launcher options after ---gpumpi:\n"
                "  -n, --numProcs N         MPI ranks\n"
                "  -g, --blocksPerGrid G    with -b: ranks = G*B when -n is absent\n"
                "  -b, --threadsPerBlock B\n"
                "  -t, --threads-per-rank T threads in each rank block (default: auto)\n"
                "  -s, --stackSize BYTES    per-thread stack (default 16K)\n"
                "  -p, --heapSize BYTES     device heap (default 1G)\n"
                "  -e, --pendingBufferSize N outstanding requests per rank (default 1024)\n"
                "  --eager-bytes BYTES      eager/rendezvous threshold (default 4096)\n"
                "  --timeout-ms MS          bound of every device wait (default 60000)\n"
                "  --out-bytes BYTES        output buffer per stream (default 16M)\n"
                "  --max-seconds S          host wall-clock limit (default none)\n"
                "  --blocks-per-rank C      each rank a cluster of C thread blocks (1, 2, 4, 8; default 1):\n"
                "                           parallel loops run on all of them\n"
                "  --one-cluster            all ranks (at most 16) in one thread-block cluster: their\n"
                "                           mailboxes live in distributed shared memory\n"
                "  -v, --verbose            launch details on stderr\n");
            exit(0);
        } else if (a == "-n" || a == "--numProcs") {
            if (!next(&v)) return -2;
            o->nranks = atoi(v.c_str());
        } else if (a == "-g" || a == "--blocksPerGrid") {
            if (!next(&v)) return -2;
            blocks = (unsigned)atoi(v.c_str());
        } else if (a == "-b" || a == "--threadsPerBlock") {
            if (!next(&v)) return -2;
            threads = (unsigned)atoi(v.c_str());
        } else if (a == "-t" || a == "--threads-per-rank") {
            if (!next(&v)) return -2;
            o->threads_per_rank = atoi(v.c_str());
        } else if (a == "-s" || a == "--stackSize") {
            if (!next(&v) || !parse_size(v.c_str(), &o->stack_bytes)) return -2;
        } else if (a == "-p" || a == "--heapSize") {
            if (!next(&v) || !parse_size(v.c_str(), &o->heap_bytes)) return -2;
        } else if (a == "-e" || a == "--pendingBufferSize") {
            if (!next(&v)) return -2;
            o->max_requests = atoi(v.c_str());
        } else if (a == "--eager-bytes") {
            if (!next(&v) || !parse_size(v.c_str(), &o->eager_bytes)) return -2;
        } else if (a == "--timeout-ms") {
            if (!next(&v)) return -2;
            o->timeout_s = atof(v.c_str()) / 1000.0;
        } else if (a == "--out-bytes") {
            if (!next(&v) || !parse_size(v.c_str(), &o->out_bytes)) return -2;
        } else if (a == "--max-seconds") {
            if (!next(&v)) return -2;
            o->max_seconds = atof(v.c_str());
        } else if (a == "--blocks-per-rank") {
            if (!next(&v)) return -2;
            o->blocks_per_rank = atoi(v.c_str());
        } else if (a == "--one-cluster") {
            o->one_cluster = 1;
        } else if (a == "-v" || a == "--verbose") {
            o->verbose = 1;
        } else {
            fprintf(stderr, "GPUMPI: unknown option '%s'\n", a.c_str());
            return -2;
        }
    }
    if (o->nranks == 0) {
        // The reference's -g/-b named blocks and threads of one-thread ranks.
        if (blocks == 0) blocks = 1;
        if (threads == 0) threads = 1;
        o->nranks = (int)(blocks * threads);
    }
    return pos;
}

namespace gm {

static double now_s() {
    timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + ts.tv_nsec * 1e-9;
}

// A kernel's cudaFuncAttributeMaxDynamicSharedMemorySize is the most dynamic
// shared memory any of its launches may use.  It only ever grows here: a size
// picked for one launch must stay allowed after a later pick for another
// launch of the same kernel tried (and set) other sizes.
static bool allow_dynamic_smem(const void* kernel, size_t smem) {
    static std::mutex mu;
    static std::map<const void*, size_t> allowed;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = allowed[kernel];
    if (smem <= 48 * 1024 || smem <= cur) return true;
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cur = smem;
    return true;
}

// ------------------------------------------------------------------ host calls
// Files the ranks of one program opened through their HostCall slots.
struct HostFiles {
    std::vector<FILE*> f;
    ~HostFiles() {
        for (FILE* fp : f)
            if (fp) fclose(fp);
    }
    FILE* get(long long h) const { return h >= 0 && h < (long long)f.size() ? f[(size_t)h] : nullptr; }
};

// Answer every posted request; returns how many were answered.
static int service_host_calls(HostCall* hc, int n, HostFiles& files) {
    int served = 0;
    for (int r = 0; r < n; r++) {
        volatile u32* state = &hc[r].state;
        if (*state != 1u) continue;
        std::atomic_thread_fence(std::memory_order_acquire);
        HostCall& c = hc[r];
        long long ret = -1;
        int err = 0;
        u32 len = 0;
        errno = 0;
        FILE* fp = files.get(c.a[0]);
        switch (c.op) {
            case HC_OPEN: {
                c.data[HOSTCALL_DATA - 1] = 0;
                const char* path = c.data;
                const size_t pl = strlen(path);
                const char* mode = pl + 1 < HOSTCALL_DATA ? c.data + pl + 1 : "r";
                FILE* nf = fopen(path, mode);
                if (nf) {
                    files.f.push_back(nf);
                    ret = (long long)files.f.size() - 1;
                }
                break;
            }
            case HC_CLOSE:
                if (fp) {
                    ret = fclose(fp) == 0 ? 0 : -1;
                    files.f[(size_t)c.a[0]] = nullptr;
                } else {
                    errno = EBADF;
                }
                break;
            case HC_WRITE:
                if (fp && c.len <= HOSTCALL_DATA) ret = (long long)fwrite(c.data, 1, c.len, fp);
                else errno = EBADF;
                break;
            case HC_READ:
                if (fp) {
                    const size_t want = c.a[1] > 0 && c.a[1] < HOSTCALL_DATA ? (size_t)c.a[1] : HOSTCALL_DATA;
                    const size_t got = fread(c.data, 1, want, fp);
                    ret = (long long)got;
                    len = (u32)got;
                } else {
                    errno = EBADF;
                }
                break;
            case HC_FLUSH:
                ret = fp && fflush(fp) == 0 ? 0 : -1;
                break;
            case HC_SEEK:
                ret = fp && fseek(fp, (long)c.a[1], (int)c.a[2]) == 0 ? 0 : -1;
                break;
            case HC_TELL:
                ret = fp ? (long long)ftell(fp) : -1;
                break;
            case HC_REMOVE:
                c.data[HOSTCALL_DATA - 1] = 0;
                ret = remove(c.data) == 0 ? 0 : -1;
                break;
            default:
                errno = ENOSYS;
                break;
        }
        if (ret < 0) err = errno ? errno : EIO;
        c.ret = ret;
        c.err = err;
        c.len = len;
        std::atomic_thread_fence(std::memory_order_release);
        *state = 2u;
        served++;
    }
    return served;
}

// Choose threads per rank: the largest of 256/128/64 that keeps every rank
// resident, given the kernel's register and shared-memory use.
size_t pick_rank_smem(const void* kernel, int T, int need) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // the largest staging area that keeps every rank block resident (a bulk
    // copy has stage bytes in flight per block)
    const size_t stages[] = {196608, 131072, 98304, 65536, 49152, 40960, 32768, 28672, 24576, 20480,
                             16384, 12288, 8192};
    for (size_t st : stages) {
        const size_t smem = rank_smem_bytes(st);
        if (!allow_dynamic_smem(kernel, smem)) continue;
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, smem) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if ((long long)per * sms >= need) return smem;
    }
    return rank_smem_bytes(0);
}

int choose_threads(const void* kernel, int n, int requested, size_t smem, int* max_resident) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int cand[] = {256, 128, 64};
    int best = 0;
    for (int k = 0; k < 3; k++) {
        int T = requested ? requested : cand[k];
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, smem) != cudaSuccess) per = 0;
        if (max_resident) *max_resident = per * sms;
        if ((long long)per * sms >= n) {
            best = T;
            break;
        }
        if (requested) break;
    }
    return best;
}

}  // namespace gm

namespace gm {

// Device image of argv: the pointer table, then the strings, with the
// pointers relocated to where the image will sit in device memory.
size_t argv_image_bytes(int argc, char** argv) {
    size_t n = sizeof(char*) * (argc + 1) + 16;
    for (int i = 0; i < argc; i++) n += strlen(argv[i]) + 1;
    return (n + 15) & ~(size_t)15;
}

void argv_image(int argc, char** argv, char* dev, std::vector<char>& img) {
    img.assign(argv_image_bytes(argc, argv), 0);
    char** ptrs = (char**)img.data();
    char* s = img.data() + sizeof(char*) * (argc + 1);
    for (int i = 0; i < argc; i++) {
        size_t l = strlen(argv[i]) + 1;
        memcpy(s, argv[i], l);
        ptrs[i] = dev + (s - img.data());
        s += l;
    }
    ptrs[argc] = nullptr;
}

// Copy a finished job's status, return values and output text back and
// derive its exit status (0 when every rank returned 0 and nothing failed).
int job_collect(HostJob& hj, cudaStream_t st, JobResult& r) {
    Job& j = hj.job;
    const int n = hj.nranks;
    u64 offs[4];
    char errmsg[256];
    r.rets.assign(n, 0);
    HCHECK(cudaMemcpyAsync(r.status, j.status, sizeof(r.status), cudaMemcpyDeviceToHost, st));
    HCHECK(cudaMemcpyAsync(offs, j.out_off, sizeof(offs), cudaMemcpyDeviceToHost, st));
    HCHECK(cudaMemcpyAsync(r.rets.data(), j.retvals, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
    HCHECK(cudaMemcpyAsync(errmsg, j.err_msg, sizeof(errmsg), cudaMemcpyDeviceToHost, st));
    HCHECK(cudaStreamSynchronize(st));
    errmsg[255] = 0;
    r.errmsg = errmsg;
    const size_t nout = offs[0] < j.out_bytes ? offs[0] : j.out_bytes;
    const size_t nerr = offs[1] < j.out_bytes ? offs[1] : j.out_bytes;
    r.out.assign(nout, 0);
    r.err.assign(nerr, 0);
    if (nout) HCHECK(cudaMemcpyAsync(&r.out[0], j.out, nout, cudaMemcpyDeviceToHost, st));
    if (nerr) HCHECK(cudaMemcpyAsync(&r.err[0], j.errout, nerr, cudaMemcpyDeviceToHost, st));
    HCHECK(cudaStreamSynchronize(st));
    r.truncated = offs[0] > j.out_bytes || offs[1] > j.out_bytes;
    r.exit_code = 0;
    r.diag.clear();
    if (r.truncated) r.diag += "GPUMPI: output truncated (raise --out-bytes)\n";
    if (r.status[1] != 0) {
        char m[400];
        snprintf(m, sizeof(m), "job failed: error %d on rank %d: %s", r.status[1], r.status[2], errmsg);
        set_last_error(m);
        r.diag += std::string("GPUMPI: ") + m + "\n";
        r.exit_code = 1;
    }
    if (r.status[3] != n) {
        char m[120];
        snprintf(m, sizeof(m), "GPUMPI: only %d of %d ranks finished\n", r.status[3], n);
        r.diag += m;
        r.exit_code = 1;
    }
    for (int q = 0; q < n; q++)
        if (r.rets[q] != 0) r.exit_code = 1;
    return GPUMPI_OK;
}

double now_seconds() { return now_s(); }

}  // namespace gm

extern "C" int gpumpi_run_program(const void* kernel, int prog_argc, char** prog_argv,
                                  const gpumpi_opts* in_opts) {
    gpumpi_opts o = *in_opts;
    opts_defaults(&o);
    const int n = o.nranks;
    if (n <= 0) {
        set_last_error("number of ranks must be positive");
        return GPUMPI_EINVAL;
    }
    const int C = o.blocks_per_rank > 0 ? o.blocks_per_rank : 1;
    if (C != 1 && C != 2 && C != 4 && C != 8) {
        set_last_error("--blocks-per-rank must be 1, 2, 4 or 8");
        fprintf(stderr, "GPUMPI: --blocks-per-rank must be 1, 2, 4 or 8\n");
        return GPUMPI_EINVAL;
    }
    const bool one = o.one_cluster != 0;
    if (one && (C != 1 || n > 16)) {
        set_last_error("--one-cluster takes at most 16 ranks of one block each");
        fprintf(stderr, "GPUMPI: --one-cluster takes at most 16 ranks of one block each\n");
        return GPUMPI_EINVAL;
    }
    int max_res = 0;
    int T = choose_threads(kernel, n * C, o.threads_per_rank, rank_smem_bytes(0), &max_res);
    if (T == 0 || T % 32 || T < 64 || T > 1024) {
        char m[256];
        snprintf(m, sizeof(m),
                 "%d ranks cannot all be resident (at most %d rank blocks of %d threads fit); "
                 "lower -t or -n",
                 n, max_res, o.threads_per_rank ? o.threads_per_rank : 64);
        set_last_error(m);
        fprintf(stderr, "GPUMPI: %s\n", m);
        return GPUMPI_ENORES;
    }
    o.threads_per_rank = T;
    size_t smem = pick_rank_smem(kernel, T, n * C);
    if (one) {
        // each block's mailbox at the end of its dynamic shared memory
        smem += MB_SMEM_BYTES;
        if (!allow_dynamic_smem(kernel, smem)) {
            set_last_error("no room for the shared-memory mailboxes");
            return GPUMPI_ENORES;
        }
        if (n > 8) HCHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    }
    if (C > 1 || one) {
        // every cluster (rank) must be resident at once
        cudaLaunchConfig_t q;
        memset(&q, 0, sizeof(q));
        q.gridDim = dim3(n * C);
        q.blockDim = dim3(T);
        q.dynamicSmemBytes = smem;
        cudaLaunchAttribute qa[1];
        qa[0].id = cudaLaunchAttributeClusterDimension;
        qa[0].val.clusterDim.x = one ? n : C;
        qa[0].val.clusterDim.y = 1;
        qa[0].val.clusterDim.z = 1;
        q.attrs = qa;
        q.numAttrs = 1;
        int clusters = 0;
        HCHECK(cudaOccupancyMaxActiveClusters(&clusters, kernel, &q));
        if (clusters < (one ? 1 : n)) {
            char m[200];
            snprintf(m, sizeof(m), "%d ranks of %d blocks cannot all be resident (at most %d clusters fit)", n, C,
                     clusters);
            set_last_error(m);
            fprintf(stderr, "GPUMPI: %s\n", m);
            return GPUMPI_ENORES;
        }
    }
    HCHECK(cudaDeviceSetLimit(cudaLimitStackSize, o.stack_bytes));

    HostJob hj;
    size_t total = host_job_layout(hj, o, n, 0, nullptr);
    char* base = nullptr;
    HCHECK(cudaMalloc(&base, total));
    host_job_layout(hj, o, n, 0, base);

    // argv in device memory
    std::vector<char> hargs;
    char* dargs = nullptr;
    HCHECK(cudaMalloc(&dargs, argv_image_bytes(prog_argc, prog_argv)));
    argv_image(prog_argc, prog_argv, dargs, hargs);
    hj.job.argc = prog_argc;
    hj.job.argv = (char**)dargs;
    hj.job.threads = T;

    // host-call slots (file I/O of the program), mapped into the device
    HostCall* hcall = nullptr;
    HCHECK(cudaHostAlloc((void**)&hcall, sizeof(HostCall) * (size_t)n, cudaHostAllocMapped));
    memset(hcall, 0, sizeof(HostCall) * (size_t)n);
    HostCall* dhcall = nullptr;
    HCHECK(cudaHostGetDevicePointer((void**)&dhcall, hcall, 0));
    hj.job.hcall = dhcall;
    HostFiles files;

    // one job, one slot per rank
    std::vector<int> slots(2 * (size_t)n);
    for (int r = 0; r < n; r++) {
        slots[r] = 0;
        slots[n + r] = r;
    }
    int* dslots = nullptr;
    HCHECK(cudaMalloc(&dslots, sizeof(int) * 2 * (size_t)n));

    cudaStream_t st;
    HCHECK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    HCHECK(cudaMemcpyAsync(dargs, hargs.data(), hargs.size(), cudaMemcpyHostToDevice, st));
    HCHECK(cudaMemcpyAsync(dslots, slots.data(), sizeof(int) * 2 * (size_t)n, cudaMemcpyHostToDevice, st));
    int rc = host_job_init(hj, st);
    if (rc) return rc;

    Launch L;
    L.jobs = (Job*)(base + hj.job_off);
    L.njobs = 1;
    L.nslots = n;
    L.slot_job = dslots;
    L.slot_rank = dslots + n;
    L.slot_base = 0;
    L.job_cluster = one ? 1 : 0;
    void* args[] = {&L};
    if (o.verbose)
        fprintf(stderr, "GPUMPI: %d ranks x %d block(s) x %d threads, job memory %.1f MiB, heap %.1f MiB\n", n, C,
                T, total / 1048576.0, o.heap_bytes / 1048576.0);
    const double t0 = now_s();
    if (C == 1 && !one) {
        HCHECK(cudaLaunchCooperativeKernel(kernel, dim3(n), dim3(T), args, smem, st));
    } else {
        cudaLaunchConfig_t cfg;
        memset(&cfg, 0, sizeof(cfg));
        cfg.gridDim = dim3(n * C);
        cfg.blockDim = dim3(T);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[2];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        at[1].id = cudaLaunchAttributeClusterDimension;
        at[1].val.clusterDim.x = one ? n : C;
        at[1].val.clusterDim.y = 1;
        at[1].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 2;
        HCHECK(cudaLaunchKernelExC(&cfg, kernel, args));
    }
    cudaEvent_t done;
    HCHECK(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    HCHECK(cudaEventRecord(done, st));
    for (;;) {
        cudaError_t q = cudaEventQuery(done);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) {
            HCHECK(q);
        }
        if (o.max_seconds > 0 && now_s() - t0 > o.max_seconds) {
            fprintf(stderr, "GPUMPI: wall-clock limit of %.1f s exceeded; ending the process\n",
                    o.max_seconds);
            fflush(stderr);
            _exit(3);
        }
        if (service_host_calls(hcall, n, files) == 0) usleep(20);
    }
    HCHECK(cudaStreamSynchronize(st));

    JobResult res;
    rc = job_collect(hj, st, res);
    if (rc) return rc;
    fwrite(res.out.data(), 1, res.out.size(), stdout);
    fflush(stdout);
    fwrite(res.err.data(), 1, res.err.size(), stderr);
    fputs(res.diag.c_str(), stderr);
    if (o.verbose) fprintf(stderr, "GPUMPI: kernel finished in %.3f s\n", now_s() - t0);
    fflush(stderr);
    cudaEventDestroy(done);
    cudaStreamDestroy(st);
    cudaFree(dslots);
    cudaFree(dargs);
    cudaFree(base);
    cudaFreeHost(hcall);
    return res.exit_code;
}
