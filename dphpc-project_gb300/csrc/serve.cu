// Serving: many MPI jobs of one program on one GPU, admitted online by HBM
// footprint into one persistent launch.
//
// The reference launches one program per process and waits for it
// (gpu_libs/gpu_main/main.cu:163-321).  Here gpumpi_server_start launches the
// program's server kernel once (server.cu: `nworkers` worker blocks, each a
// rank slot, plus an admin block) and starts a host thread that admits
// submitted jobs as soon as
//   * its job memory (mailboxes, tables, request pool, output, heap) fits in a
//     free range of one HBM pool reserved up front (first fit), and
//   * a contiguous range of idle worker blocks is free,
// in arrival order, letting a later job that fits go ahead of one that does
// not.  The host initialises an admitted job's memory with copies (copy
// engines only: the persistent launch holds the SMs) and posts an admission
// record into a ring in pinned host memory; the admin block hands the job's
// ranks to their worker blocks, which start it at once, next to the jobs
// already running (continuous batching: slots and memory freed by a finished
// job are reused by the next admitted one while others keep running).  When
// every rank of a job has finished, the admin block posts its ticket into the
// completion ring; the host thread copies the job's output and status back,
// releases its memory and slots, and hands the result to gpumpi_poll.
//
// Every job sees exactly what it would see alone (its own MPI_COMM_WORLD,
// heap and output); a converted program whose globals must start from their
// initial values should not be served twice in one process, because a rank
// slot's globals keep the values the previous rank left.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "gpumpi.h"
#include "hostjob.h"
#include "rt.cuh"

using namespace gm;

namespace {

#define SCHECK(call)                                                                  \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            char m_[400];                                                             \
            snprintf(m_, sizeof(m_), "%s failed: %s", #call, cudaGetErrorString(e_)); \
            set_last_error(m_);                                                       \
            return GPUMPI_ECUDA;                                                      \
        }                                                                             \
    } while (0)

// First-fit allocator over [0, size) in 64 KiB units.
struct RangeAlloc {
    std::vector<std::pair<size_t, size_t>> free_;   // (offset, length), sorted by offset
    explicit RangeAlloc(size_t size) { free_.push_back({0, size}); }
    bool take(size_t len, size_t* off) {
        for (size_t i = 0; i < free_.size(); i++) {
            if (free_[i].second >= len) {
                *off = free_[i].first;
                free_[i].first += len;
                free_[i].second -= len;
                if (free_[i].second == 0) free_.erase(free_.begin() + (long)i);
                return true;
            }
        }
        return false;
    }
    void give(size_t off, size_t len) {
        auto it = std::lower_bound(free_.begin(), free_.end(), std::make_pair(off, (size_t)0));
        it = free_.insert(it, {off, len});
        size_t i = (size_t)(it - free_.begin());
        if (i + 1 < free_.size() && free_[i].first + free_[i].second == free_[i + 1].first) {
            free_[i].second += free_[i + 1].second;
            free_.erase(free_.begin() + (long)i + 1);
        }
        if (i > 0 && free_[i - 1].first + free_[i - 1].second == free_[i].first) {
            free_[i - 1].second += free_[i].second;
            free_.erase(free_.begin() + (long)i);
        }
    }
};



constexpr size_t POOL_ALIGN = 64 * 1024;

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

char* dup_text(const std::string& s) {
    char* p = (char*)malloc(s.size() + 1);
    if (p) {
        memcpy(p, s.data(), s.size());
        p[s.size()] = 0;
    }
    return p;
}

}  // namespace

extern "C" void gpumpi_free(void* p) { free(p); }

namespace {

struct SJob {
    long long id = 0;
    std::vector<std::string> args;
    std::vector<char*> argv;
    int nranks = 0;
    gpumpi_opts o;
    size_t len = 0, argv_bytes = 0;
    // while admitted
    size_t off = 0;
    int slot_base = -1;
    HostJob hj;
    gpumpi_job_result res;
};

}  // namespace

struct gpumpi_server_s {
    const void* kernel = nullptr;
    gpumpi_serve_opts so;
    int T = 128, nworkers = 0;
    size_t smem = 0;
    char* pool = nullptr;
    size_t pool_bytes = 0;
    RangeAlloc* mem = nullptr;
    ServeRing* ring_h = nullptr;     // pinned host memory mapped into the device
    ServeRing* ring_d = nullptr;
    char* ctl = nullptr;             // device: worker assignments, lost flags, admin table
    int* lost_d = nullptr;
    cudaStream_t kst = nullptr, cst = nullptr;
    std::vector<char> slot_state;    // by rank slot: 0 idle, 1 running a job, 2 lost
    int nsm = 0;                     // SMs the worker blocks run on
    char* zeros = nullptr;           // pinned: sources of the job memory initialisation
    char* ones = nullptr;
    size_t fill_bytes = 0;
    std::thread thr;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<SJob*> incoming;
    std::map<long long, SJob*> finished;   // finished, not yet polled
    std::map<long long, int> known;         // 1 queued or running, 2 finished, 3 polled
    long long next_id = 1;
    bool stop_req = false, ended = false;
    int fatal = 0;
    double t0 = 0;
    u64 posted = 0, done_seen = 0;
};

namespace {

// Copy `n` bytes of the pinned fill buffer `src` (zeros or 0xff) to dst.
int fill_copy(gpumpi_server_t s, char* dst, size_t n, const char* src) {
    for (size_t o = 0; o < n; o += s->fill_bytes) {
        const size_t k = std::min(s->fill_bytes, n - o);
        SCHECK(cudaMemcpyAsync(dst + o, src, k, cudaMemcpyHostToDevice, s->cst));
    }
    return GPUMPI_OK;
}

void finish_rejected(gpumpi_server_t s, SJob* j, const char* why) {
    j->res.exit_code = 1;
    j->res.error = GPUMPI_ENORES;
    j->res.err = dup_text(why);
    j->res.start_s = j->res.end_s = now_seconds() - s->t0;
    std::lock_guard<std::mutex> g(s->mu);
    s->finished[j->id] = j;
    s->known[j->id] = 2;
    s->cv.notify_all();
}

// Admit job j if memory and contiguous idle slots are free: initialise its
// memory and post its admission record.  1 = admitted, 0 = not now, < 0 error.
int try_admit(gpumpi_server_t s, SJob* j, std::map<u64, SJob*>& running) {
    const int n = j->nranks;
    if ((int)running.size() >= SERVE_MAX_JOBS) return 0;
    int base = -1;
    for (int w = 0, run = 0; w < s->nworkers; w++) {
        run = s->slot_state[w] ? 0 : run + 1;
        if (run == n) {
            base = w - n + 1;
            break;
        }
    }
    if (base < 0) return 0;
    size_t off = 0;
    if (!s->mem->take(j->len, &off)) return 0;
    j->off = off;
    j->slot_base = base;
    char* jb = s->pool + off;
    const size_t jtotal = round_up(host_job_layout(j->hj, j->o, n, (int)(j->id & 0x7fffffff), nullptr), POOL_ALIGN);
    host_job_layout(j->hj, j->o, n, (int)(j->id & 0x7fffffff), jb);
    char* dargv = jb + jtotal;
    std::vector<char> img;
    argv_image((int)j->args.size(), j->argv.data(), dargv, img);
    j->hj.job.argc = (int)j->args.size();
    j->hj.job.argv = (char**)dargv;
    j->hj.job.threads = s->T;
    // the job's memory, by copies only: zeroed control region, all-ones page
    // lists, then the communicator headers and the job record
    int rc = fill_copy(s, j->hj.base + j->hj.zero_off, j->hj.zero_bytes, s->zeros);
    if (!rc) rc = fill_copy(s, j->hj.base + j->hj.clsp_off, j->hj.clsp_bytes, s->ones);
    if (rc) return -1;
    SCHECK(cudaMemcpyAsync(dargv, img.data(), img.size(), cudaMemcpyHostToDevice, s->cst));
    SCHECK(cudaMemcpyAsync(j->hj.job.world_cs, &j->hj.world, sizeof(CommShared), cudaMemcpyHostToDevice, s->cst));
    SCHECK(cudaMemcpyAsync(j->hj.job.self_cs, j->hj.selfs.data(), sizeof(CommShared) * j->hj.selfs.size(),
                           cudaMemcpyHostToDevice, s->cst));
    SCHECK(cudaMemcpyAsync(j->hj.base + j->hj.job_off, &j->hj.job, sizeof(Job), cudaMemcpyHostToDevice, s->cst));
    SCHECK(cudaStreamSynchronize(s->cst));
    for (int w = base; w < base + n; w++) s->slot_state[w] = 1;
    const u64 ticket = (u64)j->id;
    volatile AdmitRec* r = &s->ring_h->sub[s->posted % SERVE_RING];
    r->job = (Job*)(jb + j->hj.job_off);
    r->slot_base = base;
    r->nranks = n;
    r->ticket = ticket;
    s->posted++;
    __atomic_store_n(&s->ring_h->sub_head, s->posted, __ATOMIC_RELEASE);
    j->res.start_s = now_seconds() - s->t0;
    j->res.slot_base = base;
    running[ticket] = j;
    if (s->so.verbose)
        fprintf(stderr, "GPUMPI serve: job %lld admitted at %.3f s (%d ranks, slots %d.., %.1f MiB)\n", j->id,
                j->res.start_s, n, base, j->len / 1048576.0);
    return 1;
}

// A finished job: copy its results back, release its memory and slots.
int complete(gpumpi_server_t s, SJob* j) {
    j->res.end_s = now_seconds() - s->t0;
    JobResult jr;
    int rc = job_collect(j->hj, s->cst, jr);
    if (rc) return rc;
    std::vector<int> lost(j->nranks, 0);
    SCHECK(cudaMemcpyAsync(lost.data(), s->lost_d + j->slot_base, sizeof(int) * j->nranks, cudaMemcpyDeviceToHost,
                           s->cst));
    SCHECK(cudaStreamSynchronize(s->cst));
    j->res.exit_code = jr.exit_code;
    j->res.error = jr.status[1];
    j->res.out = dup_text(jr.out);
    j->res.err = dup_text(jr.err + jr.diag);
    s->mem->give(j->off, j->len);
    for (int r = 0; r < j->nranks; r++) s->slot_state[j->slot_base + r] = lost[r] ? 2 : 0;
    std::lock_guard<std::mutex> g(s->mu);
    s->finished[j->id] = j;
    s->known[j->id] = 2;
    s->cv.notify_all();
    return GPUMPI_OK;
}

void server_loop(gpumpi_server_t s) {
    std::vector<SJob*> waiting;   // arrival order
    std::map<u64, SJob*> running;
    int rc = GPUMPI_OK;
    for (;;) {
        bool work = false, stopping;
        {
            std::lock_guard<std::mutex> g(s->mu);
            while (!s->incoming.empty()) {
                waiting.push_back(s->incoming.front());
                s->incoming.pop_front();
            }
            stopping = s->stop_req;
        }
        for (size_t i = 0; i < waiting.size() && !rc;) {
            SJob* j = waiting[i];
            if (j->nranks <= 0 || j->nranks > s->nworkers || j->len > s->pool_bytes) {
                waiting.erase(waiting.begin() + (long)i);
                finish_rejected(s, j, j->nranks <= 0 ? "GPUMPI: job needs at least one rank\n"
                                                     : "GPUMPI: job exceeds the rank slots or the HBM pool\n");
                work = true;
                continue;
            }
            const int a = try_admit(s, j, running);
            if (a < 0) rc = GPUMPI_ECUDA;
            if (a == 1) {
                waiting.erase(waiting.begin() + (long)i);
                work = true;
            } else {
                i++;
            }
        }
        const u64 dh = __atomic_load_n(&s->ring_h->done_head, __ATOMIC_ACQUIRE);
        while (!rc && s->done_seen < dh) {
            const u64 ticket = *(volatile u64*)&s->ring_h->done[s->done_seen % SERVE_RING];
            s->done_seen++;
            auto it = running.find(ticket);
            if (it == running.end()) continue;
            SJob* j = it->second;
            running.erase(it);
            rc = complete(s, j);
            work = true;
        }
        const cudaError_t q = cudaStreamQuery(s->kst);
        if (q != cudaErrorNotReady) {
            // the persistent launch ended before it was asked to
            set_last_error(q == cudaSuccess ? "serving kernel ended early" : cudaGetErrorString(q));
            rc = GPUMPI_ECUDA;
        }
        if (rc) break;
        if (stopping && waiting.empty() && running.empty()) break;
        if (s->so.max_seconds > 0 && now_seconds() - s->t0 > s->so.max_seconds) {
            fprintf(stderr, "GPUMPI serve: wall-clock limit of %.1f s exceeded; ending the process\n",
                    s->so.max_seconds);
            fflush(stderr);
            _exit(3);
        }
        if (!work) usleep(50);
    }
    // end the persistent launch: the admin block stops once nothing runs
    __atomic_store_n(&s->ring_h->stop, 1, __ATOMIC_RELEASE);
    if (rc) __atomic_store_n(&s->ring_h->kill, 1, __ATOMIC_RELEASE);
    const cudaError_t e = cudaStreamSynchronize(s->kst);
    if (!rc && e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        rc = GPUMPI_ECUDA;
    }
    // jobs that never ran (or were cut short by a failure) report it
    for (SJob* j : waiting) finish_rejected(s, j, "GPUMPI: the server ended before the job ran\n");
    for (auto& kv : running) finish_rejected(s, kv.second, "GPUMPI: the server failed while the job ran\n");
    std::lock_guard<std::mutex> g(s->mu);
    s->fatal = rc;
    s->ended = true;
    s->cv.notify_all();
}

}  // namespace

extern "C" int gpumpi_server_start(const void* kernel, const gpumpi_serve_opts* sopts, gpumpi_server_t* out) {
    if (!kernel || !sopts || !out) {
        set_last_error("gpumpi_server_start: bad arguments");
        return GPUMPI_EINVAL;
    }
    gpumpi_serve_opts so = *sopts;
    const int T = so.threads_per_rank ? so.threads_per_rank : 128;
    if (T < 64 || T > 1024 || T % 32) {
        set_last_error("gpumpi_server_start: threads_per_rank must be 64..1024, a multiple of 32");
        return GPUMPI_EINVAL;
    }
    if (so.timeout_s <= 0) so.timeout_s = 60.0;
    int dev = 0, sms = 0, per = 0;
    SCHECK(cudaGetDevice(&dev));
    SCHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, rank_smem_bytes(0)));
    int capacity = per * sms;   // worker blocks + the admin block
    if (capacity > 1025) capacity = 1025;
    const int want = so.max_slots > 0 && so.max_slots + 1 < capacity ? so.max_slots + 1 : capacity;
    const size_t smem = pick_rank_smem(kernel, T, want);
    SCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, smem));
    const int nblocks = std::min(want, per * sms);
    if (nblocks < 2) {
        set_last_error("gpumpi_server_start: no room for a worker block");
        return GPUMPI_ENORES;
    }
    gpumpi_server_t s = new gpumpi_server_s();
    s->kernel = kernel;
    s->so = so;
    s->T = T;
    s->smem = smem;
    s->nworkers = nblocks - 1;
    s->slot_state.assign(s->nworkers, 0);
    size_t pool_bytes = so.pool_bytes;
    if (pool_bytes == 0) {
        size_t fr = 0, tot = 0;
        SCHECK(cudaMemGetInfo(&fr, &tot));
        pool_bytes = fr / 2;
    }
    s->pool_bytes = round_up(pool_bytes, POOL_ALIGN);
    SCHECK(cudaMalloc(&s->pool, s->pool_bytes));
    s->mem = new RangeAlloc(s->pool_bytes);
    SCHECK(cudaHostAlloc((void**)&s->ring_h, sizeof(ServeRing), cudaHostAllocMapped));
    memset((void*)s->ring_h, 0, sizeof(ServeRing));
    SCHECK(cudaHostGetDevicePointer((void**)&s->ring_d, s->ring_h, 0));
    s->fill_bytes = (size_t)4 << 20;
    SCHECK(cudaHostAlloc((void**)&s->zeros, s->fill_bytes, cudaHostAllocDefault));
    SCHECK(cudaHostAlloc((void**)&s->ones, s->fill_bytes, cudaHostAllocDefault));
    memset(s->zeros, 0, s->fill_bytes);
    memset(s->ones, 0xff, s->fill_bytes);
    const size_t W = (size_t)s->nworkers;
    const size_t o_seq = 0, o_job = o_seq + 8 * W, o_rank = o_job + 8 * W, o_lost = o_rank + 4 * W;
    const size_t o_slot = o_lost + 4 * W, o_sm = o_slot + 4 * W, o_perm = o_sm + 4 * W;
    const size_t o_act = round_up(o_perm + 4 * W, 256);
    const size_t ctl_bytes = o_act + sizeof(ServeActive) * SERVE_MAX_JOBS;
    SCHECK(cudaMalloc(&s->ctl, ctl_bytes));
    SCHECK(cudaMemset(s->ctl, 0, ctl_bytes));
    SCHECK(cudaMemset(s->ctl + o_sm, 0xff, 4 * W));   // -1 until each worker reports its SM
    s->lost_d = (int*)(s->ctl + o_lost);
    SCHECK(cudaStreamCreateWithFlags(&s->kst, cudaStreamNonBlocking));
    SCHECK(cudaStreamCreateWithFlags(&s->cst, cudaStreamNonBlocking));
    size_t stack = 16 * 1024;
    SCHECK(cudaDeviceSetLimit(cudaLimitStackSize, stack));
    SCHECK(cudaDeviceSynchronize());
    ServerArgs A;
    A.ring = s->ring_d;
    A.assign_seq = (u64*)(s->ctl + o_seq);
    A.assign_job = (Job**)(s->ctl + o_job);
    A.assign_rank = (int*)(s->ctl + o_rank);
    A.assign_slot = (int*)(s->ctl + o_slot);
    A.worker_sm = (int*)(s->ctl + o_sm);
    A.perm = (const int*)(s->ctl + o_perm);
    A.lost = s->lost_d;
    A.active = (ServeActive*)(s->ctl + o_act);
    A.nworkers = s->nworkers;
    A.slot_base = 0;
    void* args[] = {&A};
    SCHECK(cudaLaunchCooperativeKernel(kernel, dim3(nblocks), dim3(T), args, smem, s->kst));
    // Rank slots over worker blocks: every worker reports its SM, then slot k
    // goes to the (k / nsm)-th worker of the (k mod nsm)-th SM, so that the
    // consecutive slots of one job lie on different SMs.  Until the map is in
    // device memory no job is admitted (the admin block reads it only then).
    {
        std::vector<int> sm(W, -1);
        const double tw = now_seconds();
        for (;;) {
            SCHECK(cudaMemcpyAsync(sm.data(), s->ctl + o_sm, 4 * W, cudaMemcpyDeviceToHost, s->cst));
            SCHECK(cudaStreamSynchronize(s->cst));
            if (std::find(sm.begin(), sm.end(), -1) == sm.end()) break;
            if (now_seconds() - tw > 30.0) {
                set_last_error("gpumpi_server_start: worker blocks did not start");
                __atomic_store_n(&s->ring_h->kill, 1, __ATOMIC_RELEASE);
                cudaStreamSynchronize(s->kst);
                return GPUMPI_ECUDA;
            }
            usleep(100);
        }
        std::map<int, std::vector<int>> by_sm;
        for (size_t w = 0; w < W; w++) by_sm[sm[w]].push_back((int)w);
        std::vector<int> perm;
        for (size_t layer = 0; perm.size() < W; layer++)
            for (auto& kv : by_sm)
                if (layer < kv.second.size()) perm.push_back(kv.second[layer]);
        SCHECK(cudaMemcpyAsync(s->ctl + o_perm, perm.data(), 4 * W, cudaMemcpyHostToDevice, s->cst));
        SCHECK(cudaStreamSynchronize(s->cst));
        s->nsm = (int)by_sm.size();
    }
    s->t0 = now_seconds();
    if (so.verbose)
        fprintf(stderr, "GPUMPI serve: %d worker blocks of %d threads, pool %.1f MiB\n", s->nworkers, T,
                s->pool_bytes / 1048576.0);
    s->thr = std::thread(server_loop, s);
    *out = s;
    return GPUMPI_OK;
}

extern "C" int gpumpi_submit(gpumpi_server_t s, const gpumpi_job_spec* spec, long long* job_id) {
    if (!s || !spec || spec->argc < 0 || (spec->argc && !spec->argv)) {
        set_last_error("gpumpi_submit: bad arguments");
        return GPUMPI_EINVAL;
    }
    SJob* j = new SJob();
    for (int i = 0; i < spec->argc; i++) j->args.push_back(spec->argv[i] ? spec->argv[i] : "");
    for (auto& a : j->args) j->argv.push_back((char*)a.c_str());
    j->argv.push_back(nullptr);
    j->nranks = spec->nranks;
    memset(&j->o, 0, sizeof(j->o));
    j->o.nranks = spec->nranks;
    j->o.heap_bytes = spec->heap_bytes ? spec->heap_bytes : ((size_t)256 << 20);
    j->o.timeout_s = s->so.timeout_s;
    j->o.threads_per_rank = s->T;
    opts_defaults(&j->o);
    const int n = spec->nranks > 0 ? spec->nranks : 1;
    j->argv_bytes = argv_image_bytes((int)j->args.size(), j->argv.data());
    j->len = round_up(round_up(job_footprint(j->o, n), POOL_ALIGN) + round_up(j->argv_bytes, 256), POOL_ALIGN);
    memset(&j->res, 0, sizeof(j->res));
    j->res.footprint = j->len;
    j->res.slot_base = -1;
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop_req || s->ended) {
        delete j;
        set_last_error("gpumpi_submit: the server is stopping");
        return GPUMPI_EINVAL;
    }
    j->id = s->next_id++;
    j->res.submit_s = now_seconds() - s->t0;
    s->known[j->id] = 1;
    s->incoming.push_back(j);
    if (job_id) *job_id = j->id;
    return GPUMPI_OK;
}

extern "C" int gpumpi_poll(gpumpi_server_t s, long long job_id, int wait_ms, gpumpi_job_result* result) {
    if (!s || !result) return GPUMPI_EINVAL;
    std::unique_lock<std::mutex> g(s->mu);
    auto k = s->known.find(job_id);
    if (k == s->known.end() || k->second == 3) {
        set_last_error("gpumpi_poll: unknown job, or its result was already returned");
        return GPUMPI_EINVAL;
    }
    auto ready = [&]() { return s->finished.count(job_id) > 0; };
    if (!ready()) {
        if (wait_ms < 0) s->cv.wait(g, [&]() { return ready() || s->ended; });
        else if (wait_ms > 0) s->cv.wait_for(g, std::chrono::milliseconds(wait_ms), [&]() { return ready() || s->ended; });
    }
    if (!ready()) return GPUMPI_EAGAIN;
    SJob* j = s->finished[job_id];
    s->finished.erase(job_id);
    s->known[job_id] = 3;
    *result = j->res;   // the texts now belong to the caller (gpumpi_free)
    delete j;
    return GPUMPI_OK;
}

extern "C" int gpumpi_server_stop(gpumpi_server_t s) {
    if (!s) return GPUMPI_EINVAL;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop_req = true;
    }
    if (s->thr.joinable()) s->thr.join();
    const int rc = s->fatal;
    for (auto& kv : s->finished) {
        gpumpi_free(kv.second->res.out);
        gpumpi_free(kv.second->res.err);
        delete kv.second;
    }
    cudaStreamDestroy(s->kst);
    cudaStreamDestroy(s->cst);
    cudaFree(s->ctl);
    cudaFree(s->pool);
    cudaFreeHost(s->ring_h);
    cudaFreeHost(s->zeros);
    cudaFreeHost(s->ones);
    delete s->mem;
    delete s;
    return rc;
}

// The whole list of jobs, each submitted at its arrival time.
extern "C" int gpumpi_serve(const void* kernel, const gpumpi_job_spec* jobs, int njobs,
                            const gpumpi_serve_opts* sopts, gpumpi_job_result* results) {
    if (!kernel || njobs < 0 || (njobs && (!jobs || !results)) || !sopts) {
        set_last_error("gpumpi_serve: bad arguments");
        return GPUMPI_EINVAL;
    }
    gpumpi_server_t s = nullptr;
    int rc = gpumpi_server_start(kernel, sopts, &s);
    if (rc) return rc;
    std::vector<int> order(njobs);
    for (int k = 0; k < njobs; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].submit_s < jobs[b].submit_s; });
    std::vector<long long> ids(njobs, 0);
    std::vector<double> arrive(njobs, 0.0);
    for (int k : order) {
        const double wait = jobs[k].submit_s - (now_seconds() - s->t0);
        if (wait > 0) usleep((useconds_t)(wait * 1e6));
        rc = gpumpi_submit(s, &jobs[k], &ids[k]);
        if (rc) break;
        arrive[k] = jobs[k].submit_s;
    }
    int rc_all = rc;
    for (int k = 0; k < njobs && !rc; k++) {
        int prc = gpumpi_poll(s, ids[k], -1, &results[k]);
        if (prc) {
            rc_all = prc;
            memset(&results[k], 0, sizeof(results[k]));
            results[k].exit_code = 1;
            results[k].slot_base = -1;
            continue;
        }
        results[k].submit_s = arrive[k];   // the requested arrival (the submit ran then)
        if (results[k].exit_code) rc_all = rc_all ? rc_all : GPUMPI_EJOB;
    }
    const int src = gpumpi_server_stop(s);
    return src ? src : rc_all;
}

namespace {

void print_job(size_t k, int nranks, const gpumpi_job_result& r) {
    std::istringstream os(r.out ? r.out : "");
    std::string l;
    while (std::getline(os, l)) printf("[job %zu] %s\n", k, l.c_str());
    if (r.err && *r.err) fprintf(stderr, "[job %zu] %s", k, r.err);
    printf("serve job %zu ranks %d exit %d slots %d footprint_mib %.1f submit %.6f start %.6f end %.6f "
           "latency %.6f\n",
           k, nranks, r.exit_code, r.slot_base, r.footprint / 1048576.0, r.submit_s, r.start_s, r.end_s,
           r.end_s - r.submit_s);
}

void print_summary(std::vector<double> lat, double makespan) {
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)(q * (double)(lat.size() - 1) + 0.5);
        return lat[std::min(i, lat.size() - 1)];
    };
    printf("serve summary jobs %zu makespan %.6f latency_p50 %.6f latency_p99 %.6f\n", lat.size(), makespan,
           pct(0.50), pct(0.99));
    fflush(stdout);
}

// Jobs from standard input, submitted as their lines arrive; results printed
// as the jobs finish.
int serve_stream(const void* kernel, const gpumpi_serve_opts& so, size_t heap, char* prog) {
    gpumpi_server_t s = nullptr;
    if (gpumpi_server_start(kernel, &so, &s) != GPUMPI_OK) {
        fprintf(stderr, "GPUMPI serve: %s\n", gpumpi_last_error());
        return 1;
    }
    struct Pending {
        long long id;
        size_t k;
        int nranks;
    };
    std::vector<Pending> pending;
    std::vector<double> lat;
    double makespan = 0.0;
    int status = 0;
    auto drain = [&](int wait_ms) {
        for (size_t i = 0; i < pending.size();) {
            gpumpi_job_result r;
            const int rc = gpumpi_poll(s, pending[i].id, wait_ms, &r);
            if (rc == GPUMPI_EAGAIN) {
                i++;
                continue;
            }
            if (rc != GPUMPI_OK) {
                status = 1;
                pending.erase(pending.begin() + (long)i);
                continue;
            }
            print_job(pending[i].k, pending[i].nranks, r);
            fflush(stdout);
            lat.push_back(r.end_s - r.submit_s);
            makespan = std::max(makespan, r.end_s);
            if (r.exit_code) status = 1;
            gpumpi_free(r.out);
            gpumpi_free(r.err);
            pending.erase(pending.begin() + (long)i);
        }
    };
    std::mutex mu;
    std::vector<std::string> lines;
    bool eof = false;
    std::thread reader([&]() {
        std::string line;
        while (std::getline(std::cin, line)) {
            std::lock_guard<std::mutex> g(mu);
            lines.push_back(line);
        }
        std::lock_guard<std::mutex> g(mu);
        eof = true;
    });
    size_t k = 0;
    for (;;) {
        std::vector<std::string> got;
        bool done;
        {
            std::lock_guard<std::mutex> g(mu);
            got.swap(lines);
            done = eof;
        }
        for (std::string line : got) {
            const size_t h = line.find('#');
            if (h != std::string::npos) line.resize(h);
            std::istringstream ls(line);
            std::vector<std::string> w;
            std::string t;
            while (ls >> t) w.push_back(t);
            if (w.size() < 2) continue;
            std::vector<char*> av;
            av.push_back(prog);
            for (size_t q = 2; q < w.size(); q++) av.push_back((char*)w[q].c_str());
            av.push_back(nullptr);
            gpumpi_job_spec spec;
            memset(&spec, 0, sizeof(spec));
            spec.nranks = atoi(w[0].c_str());
            spec.heap_bytes = heap;
            spec.argc = (int)av.size() - 1;
            spec.argv = av.data();
            long long id = 0;
            if (gpumpi_submit(s, &spec, &id) != GPUMPI_OK) {
                fprintf(stderr, "GPUMPI serve: %s\n", gpumpi_last_error());
                status = 1;
                continue;
            }
            pending.push_back({id, k++, spec.nranks});
        }
        drain(0);
        if (done && got.empty()) break;
        usleep(200);
    }
    reader.join();
    while (!pending.empty()) drain(50);
    if (gpumpi_server_stop(s) != GPUMPI_OK) status = 1;
    print_summary(lat, makespan);
    return status;
}

}  // namespace

// Command line: "<prog> ---gpumpi --serve JOBFILE [--pool BYTES] [--max-slots N]
// [-t T] [-p HEAP] [--timeout-ms MS] [--max-seconds S] [-v]".  Each JOBFILE line
// is "<ranks> <arrival-ms> [program arguments...]"; '#' starts a comment.
// Prints every job's output prefixed with "[job k] " in job order, one
// "serve job" line per job with its times, and a summary with the makespan and
// the 50th/99th percentile of the job latency (arrival to end).  With
// "--serve -" the lines come from standard input: each job is submitted when
// its line is read and its output and "serve job" line are printed as soon as
// it finishes (in completion order); end of input ends the server once the
// submitted jobs have finished.
extern "C" int gpumpi_serve_main(const void* kernel, int argc, char** argv) {
    int pos = -1;
    for (int i = 1; i < argc; i++)
        if (strcmp(argv[i], "---gpumpi") == 0) {
            pos = i;
            break;
        }
    if (pos < 0) return 1;
    std::string file;
    gpumpi_serve_opts so;
    memset(&so, 0, sizeof(so));
    size_t heap = 0;
    std::vector<char*> rest;
    rest.push_back(argv[0]);
    rest.push_back(argv[pos]);
    auto size_arg = [](const char* s) {
        char* e = nullptr;
        double v = strtod(s, &e);
        if (*e == 'k' || *e == 'K') v *= 1024.0;
        else if (*e == 'm' || *e == 'M') v *= 1048576.0;
        else if (*e == 'g' || *e == 'G') v *= 1073741824.0;
        return (size_t)v;
    };
    for (int i = pos + 1; i < argc; i++) {
        std::string a = argv[i];
        auto val = [&]() -> const char* { return i + 1 < argc ? argv[++i] : ""; };
        if (a == "--serve") file = val();
        else if (a == "--pool") so.pool_bytes = size_arg(val());
        else if (a == "--max-slots") so.max_slots = atoi(val());
        else if (a == "-t" || a == "--threads-per-rank") so.threads_per_rank = atoi(val());
        else if (a == "-p" || a == "--heapSize") heap = size_arg(val());
        else if (a == "--timeout-ms") so.timeout_s = atof(val()) / 1000.0;
        else if (a == "--max-seconds") so.max_seconds = atof(val());
        else if (a == "-v" || a == "--verbose") so.verbose = 1;
        else {
            fprintf(stderr, "GPUMPI serve: unknown option '%s'\n", a.c_str());
            return 1;
        }
    }
    if (file == "-") return serve_stream(kernel, so, heap, argv[0]);
    std::ifstream in(file);
    if (!in) {
        fprintf(stderr, "GPUMPI serve: cannot read job file '%s'\n", file.c_str());
        return 1;
    }
    std::vector<gpumpi_job_spec> specs;
    std::vector<std::vector<std::string>> words;
    std::string line;
    while (std::getline(in, line)) {
        const size_t h = line.find('#');
        if (h != std::string::npos) line.resize(h);
        std::istringstream ls(line);
        std::vector<std::string> w;
        std::string t;
        while (ls >> t) w.push_back(t);
        if (w.size() < 2) continue;
        words.push_back(w);
    }
    std::vector<std::vector<char*>> jargv(words.size());
    for (size_t k = 0; k < words.size(); k++) {
        gpumpi_job_spec s;
        memset(&s, 0, sizeof(s));
        s.nranks = atoi(words[k][0].c_str());
        s.submit_s = atof(words[k][1].c_str()) / 1000.0;
        s.heap_bytes = heap;
        jargv[k].push_back(argv[0]);
        for (size_t q = 2; q < words[k].size(); q++) jargv[k].push_back((char*)words[k][q].c_str());
        s.argc = (int)jargv[k].size();
        jargv[k].push_back(nullptr);
        s.argv = jargv[k].data();
        specs.push_back(s);
    }
    std::vector<gpumpi_job_result> res(specs.size());
    const int rc = gpumpi_serve(kernel, specs.data(), (int)specs.size(), &so, res.data());
    if (rc != GPUMPI_OK && rc != GPUMPI_EJOB) {
        fprintf(stderr, "GPUMPI serve: %s\n", gpumpi_last_error());
        return 1;
    }
    std::vector<double> lat;
    double makespan = 0.0;
    int status = 0;
    for (size_t k = 0; k < res.size(); k++) {
        const gpumpi_job_result& r = res[k];
        print_job(k, specs[k].nranks, r);
        lat.push_back(r.end_s - r.submit_s);
        makespan = std::max(makespan, r.end_s);
        if (r.exit_code) status = 1;
        gpumpi_free(r.out);
        gpumpi_free(r.err);
    }
    print_summary(lat, makespan);
    return status;
}
