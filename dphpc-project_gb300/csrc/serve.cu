// Serving: many MPI jobs of one program on one GPU, admitted by HBM footprint.
//
// The reference launches one program per process and waits for it
// (gpu_libs/gpu_main/main.cu:163-321).  Here a host loop keeps a queue of
// jobs (rank count, arguments, arrival time) and admits a job as soon as
//   * its job memory (mailboxes, tables, request pool, output, heap) fits in a
//     free range of one HBM pool reserved up front (first fit), and
//   * a contiguous range of rank slots is free, with the running ranks never
//     exceeding the rank blocks the GPU holds at once,
// in arrival order, letting a later job that fits go ahead of one that does
// not.  Each admitted job is one cooperative launch on its own stream, so the
// jobs run side by side as separate kernels; because the running ranks always
// fit on the GPU together, a job's ranks are co-resident even while other jobs
// run, and no job waits on another.  A job's slot range keeps its ranks'
// converted globals apart from every other running job's.  When a job's
// kernel ends, its output and status are copied back on its stream and its
// pool range and slots are released.
//
// Every job sees exactly what it would see alone (its own MPI_COMM_WORLD,
// heap and output); a converted program whose globals must start from their
// initial values should not be served twice in one process, because device
// globals keep their values between launches.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <algorithm>
#include <fstream>
#include <sstream>
#include <string>
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

struct Running {
    int job;
    size_t off, len;
    size_t slot_off;
    int slot_base;
    HostJob hj;
    cudaStream_t st;
    cudaEvent_t done;
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

extern "C" int gpumpi_serve(const void* kernel, const gpumpi_job_spec* jobs, int njobs,
                            const gpumpi_serve_opts* sopts, gpumpi_job_result* results) {
    if (!kernel || njobs < 0 || (njobs && (!jobs || !results)) || !sopts) {
        set_last_error("gpumpi_serve: bad arguments");
        return GPUMPI_EINVAL;
    }
    gpumpi_serve_opts so = *sopts;
    const int T = so.threads_per_rank ? so.threads_per_rank : 128;
    if (T < 64 || T > 1024 || T % 32) {
        set_last_error("gpumpi_serve: threads_per_rank must be 64..1024, a multiple of 32");
        return GPUMPI_EINVAL;
    }
    int dev = 0, sms = 0, per = 0;
    SCHECK(cudaGetDevice(&dev));
    SCHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, rank_smem_bytes(0)));
    int capacity = per * sms;
    if (capacity > 1024) capacity = 1024;
    // every rank that may run at once keeps its staging area: size it for the capacity
    const size_t smem = pick_rank_smem(kernel, T, so.max_slots > 0 && so.max_slots < capacity ? so.max_slots : capacity);
    SCHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, T, smem));
    if (per * sms < capacity) capacity = per * sms;
    const int max_slots = so.max_slots > 0 && so.max_slots < capacity ? so.max_slots : capacity;
    size_t pool_bytes = so.pool_bytes;
    if (pool_bytes == 0) {
        size_t fr = 0, tot = 0;
        SCHECK(cudaMemGetInfo(&fr, &tot));
        pool_bytes = fr / 2;
    }
    pool_bytes = round_up(pool_bytes, POOL_ALIGN);

    // per-job options and footprints
    std::vector<gpumpi_opts> jopts(njobs);
    std::vector<size_t> jlen(njobs), jargv(njobs);
    size_t stack = 16 * 1024;
    for (int k = 0; k < njobs; k++) {
        gpumpi_opts o;
        memset(&o, 0, sizeof(o));
        o.nranks = jobs[k].nranks;
        o.heap_bytes = jobs[k].heap_bytes ? jobs[k].heap_bytes : ((size_t)256 << 20);
        o.timeout_s = so.timeout_s;
        o.threads_per_rank = T;
        opts_defaults(&o);
        if (o.stack_bytes > stack) stack = o.stack_bytes;
        jopts[k] = o;
        const int n = o.nranks > 0 ? o.nranks : 1;
        jargv[k] = argv_image_bytes(jobs[k].argc, jobs[k].argv);
        jlen[k] = round_up(job_footprint(o, n), POOL_ALIGN) + round_up(jargv[k], 256) +
                  round_up(sizeof(int) * 2 * (size_t)n, 256);
        jlen[k] = round_up(jlen[k], POOL_ALIGN);
        memset(&results[k], 0, sizeof(results[k]));
        results[k].footprint = jlen[k];
        results[k].submit_s = jobs[k].submit_s;
        results[k].slot_base = -1;
    }
    SCHECK(cudaDeviceSetLimit(cudaLimitStackSize, stack));
    char* pool = nullptr;
    SCHECK(cudaMalloc(&pool, pool_bytes));
    RangeAlloc mem(pool_bytes);
    std::vector<char> slot_used(max_slots, 0);
    int slots_in_use = 0;

    std::vector<int> state(njobs, 0);   // 0 waiting, 1 running, 2 finished
    std::vector<Running> run;
    int finished = 0, rc_all = GPUMPI_OK;
    for (int k = 0; k < njobs; k++) {
        if (jobs[k].nranks <= 0 || jobs[k].nranks > max_slots || jlen[k] > pool_bytes) {
            results[k].exit_code = 1;
            results[k].error = GPUMPI_ENORES;
            results[k].err = dup_text(jobs[k].nranks <= 0 ? "GPUMPI: job needs at least one rank\n"
                                                          : "GPUMPI: job exceeds the rank slots or the HBM pool\n");
            state[k] = 2;
            finished++;
        }
    }
    const double t0 = now_seconds();
    std::vector<char> img;
    while (finished < njobs) {
        const double now = now_seconds() - t0;
        // admission, in arrival order
        std::vector<int> order;
        for (int k = 0; k < njobs; k++)
            if (state[k] == 0 && jobs[k].submit_s <= now) order.push_back(k);
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return jobs[a].submit_s < jobs[b].submit_s; });
        for (int k : order) {
            const int n = jobs[k].nranks;
            if (slots_in_use + n > max_slots) continue;
            int base = -1;
            for (int s = 0, runlen = 0; s < max_slots; s++) {
                runlen = slot_used[s] ? 0 : runlen + 1;
                if (runlen == n) {
                    base = s - n + 1;
                    break;
                }
            }
            if (base < 0) continue;
            size_t off = 0;
            if (!mem.take(jlen[k], &off)) continue;
            Running R;
            R.job = k;
            R.off = off;
            R.len = jlen[k];
            R.slot_base = base;
            char* jb = pool + off;
            const size_t jtotal = round_up(host_job_layout(R.hj, jopts[k], n, k, nullptr), POOL_ALIGN);
            host_job_layout(R.hj, jopts[k], n, k, jb);
            char* dargv = jb + jtotal;
            int* dslots = (int*)(dargv + round_up(jargv[k], 256));
            argv_image(jobs[k].argc, jobs[k].argv, dargv, img);
            R.hj.job.argc = jobs[k].argc;
            R.hj.job.argv = (char**)dargv;
            R.hj.job.threads = T;
            std::vector<int> slots(2 * (size_t)n);
            for (int q = 0; q < n; q++) {
                slots[q] = 0;
                slots[n + q] = q;
            }
            SCHECK(cudaStreamCreateWithFlags(&R.st, cudaStreamNonBlocking));
            SCHECK(cudaEventCreateWithFlags(&R.done, cudaEventDisableTiming));
            SCHECK(cudaMemcpyAsync(dargv, img.data(), img.size(), cudaMemcpyHostToDevice, R.st));
            SCHECK(cudaMemcpyAsync(dslots, slots.data(), sizeof(int) * slots.size(), cudaMemcpyHostToDevice, R.st));
            int rc = host_job_init(R.hj, R.st);
            if (rc) return rc;
            // the host images above must stay valid until the copies ran
            SCHECK(cudaStreamSynchronize(R.st));
            Launch L;
            L.jobs = (Job*)(jb + R.hj.job_off);
            L.njobs = 1;
            L.nslots = n;
            L.slot_job = dslots;
            L.slot_rank = dslots + n;
            L.slot_base = base;
            void* args[] = {&L};
            results[k].start_s = now_seconds() - t0;
            results[k].slot_base = base;
            SCHECK(cudaLaunchCooperativeKernel(kernel, dim3(n), dim3(T), args, smem, R.st));
            SCHECK(cudaEventRecord(R.done, R.st));
            for (int s = base; s < base + n; s++) slot_used[s] = 1;
            slots_in_use += n;
            state[k] = 1;
            if (so.verbose)
                fprintf(stderr, "GPUMPI serve: job %d admitted at %.3f s (%d ranks, slots %d.., %.1f MiB)\n", k,
                        results[k].start_s, n, base, jlen[k] / 1048576.0);
            run.push_back(R);
        }
        // completions
        bool progressed = false;
        for (size_t i = 0; i < run.size();) {
            cudaError_t q = cudaEventQuery(run[i].done);
            if (q == cudaErrorNotReady) {
                i++;
                continue;
            }
            Running R = run[i];
            run.erase(run.begin() + (long)i);
            const int k = R.job;
            results[k].end_s = now_seconds() - t0;
            if (q != cudaSuccess) {
                set_last_error(cudaGetErrorString(q));
                return GPUMPI_ECUDA;
            }
            JobResult jr;
            int rc = job_collect(R.hj, R.st, jr);
            if (rc) return rc;
            results[k].exit_code = jr.exit_code;
            results[k].error = jr.status[1];
            results[k].out = dup_text(jr.out);
            results[k].err = dup_text(jr.err + jr.diag);
            if (jr.exit_code) rc_all = GPUMPI_EJOB;
            cudaEventDestroy(R.done);
            cudaStreamDestroy(R.st);
            mem.give(R.off, R.len);
            for (int s = R.slot_base; s < R.slot_base + jobs[k].nranks; s++) slot_used[s] = 0;
            slots_in_use -= jobs[k].nranks;
            state[k] = 2;
            finished++;
            progressed = true;
        }
        if (so.max_seconds > 0 && now_seconds() - t0 > so.max_seconds) {
            fprintf(stderr, "GPUMPI serve: wall-clock limit of %.1f s exceeded; ending the process\n",
                    so.max_seconds);
            fflush(stderr);
            _exit(3);
        }
        if (!progressed) usleep(100);
    }
    cudaFree(pool);
    return rc_all;
}

// Command line: "<prog> ---gpumpi --serve JOBFILE [--pool BYTES] [--max-slots N]
// [-t T] [-p HEAP] [--timeout-ms MS] [--max-seconds S] [-v]".  Each JOBFILE line
// is "<ranks> <arrival-ms> [program arguments...]"; '#' starts a comment.
// Prints every job's output prefixed with "[job k] " in job order, one
// "serve job" line per job with its times, and a summary with the makespan and
// the 50th/99th percentile of the job latency (arrival to end).
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
        std::istringstream os(r.out ? r.out : "");
        std::string l;
        while (std::getline(os, l)) printf("[job %zu] %s\n", k, l.c_str());
        if (r.err && *r.err) fprintf(stderr, "[job %zu] %s", k, r.err);
        printf("serve job %zu ranks %d exit %d slots %d footprint_mib %.1f submit %.6f start %.6f end %.6f "
               "latency %.6f\n",
               k, specs[k].nranks, r.exit_code, r.slot_base, r.footprint / 1048576.0, r.submit_s, r.start_s, r.end_s,
               r.end_s - r.submit_s);
        lat.push_back(r.end_s - r.submit_s);
        makespan = std::max(makespan, r.end_s);
        if (r.exit_code) status = 1;
        gpumpi_free(r.out);
        gpumpi_free(r.err);
    }
    std::sort(lat.begin(), lat.end());
    auto pct = [&](double q) {
        if (lat.empty()) return 0.0;
        size_t i = (size_t)(q * (double)(lat.size() - 1) + 0.5);
        return lat[std::min(i, lat.size() - 1)];
    };
    printf("serve summary jobs %zu makespan %.6f latency_p50 %.6f latency_p99 %.6f\n", res.size(), makespan,
           pct(0.50), pct(0.99));
    fflush(stdout);
    return status;
}
