// Autotuner for the host-driven collectives.
//
// Plain form: for every distinct descriptor shape (collective, type,
// operator, ranks, count) it times each candidate schedule (the descriptor's
// `algo`) at each thread count whose rank blocks are co-resident, as a plain
// launch of that descriptor alone.  Batched form: a schedule that wins alone
// at 1024 threads may lose at the 128 threads of a 1024-rank launch and next
// to fifteen other communicators, so the batched choice is measured in the
// batched launch itself: for each co-resident thread count, every descriptor
// takes its best schedule at that count, the whole list is timed, and at the
// winning count each (collective, type) group tries every schedule in turn,
// then flag rounds for its calls (`sync`) in a launch-ordered plan.
// Timing: two untimed launches, then `reps` launches between CUDA events on
// a stream of its own.  Plain results are cached, one line per shape, thread
// count and GPU:
//   <gpu name>|<op> <dtype> <redop> <ranks> <count> <threads>|<algo> <us>
// so a later run with the same shapes skips those measurements.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gpumpi.h"
#include "hostjob.h"

using namespace gm;

namespace {

struct Choice {
    int algo = 0;
    double us = -1.0;   // < 0: not co-resident at this thread count
};

const int kThreads[] = {64, 128, 256, 512, 1024};
constexpr int kNT = 5;

std::string shape_key(const gpumpi_coll_desc& d) {
    int n = 0;
    gpumpi_comm_size(d.comm, &n);
    std::ostringstream k;
    k << d.op << ' ' << d.dtype << ' ' << d.redop << ' ' << n << ' ' << d.count;
    return k.str();
}

std::vector<int> algos_of(int op) {
    switch (op) {
        case GPUMPI_COLL_BCAST: return {1, 2};
        case GPUMPI_COLL_REDUCE: return {1, 2};
        case GPUMPI_COLL_ALLREDUCE: return {1, 2, 3};
        case GPUMPI_COLL_ALLTOALL:
        case GPUMPI_COLL_ALLGATHER: return {1, 2, 3, 4};
        default: return {0};
    }
}

// Average microseconds per launch of a plan (its error status checked after).
int time_plan(gpumpi_plan_t plan, int reps, cudaStream_t st, double* us) {
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return GPUMPI_ECUDA;
    int rc = GPUMPI_OK;
    for (int i = 0; i < 2 && !rc; i++) rc = gpumpi_plan_launch(plan, st);
    if (!rc && cudaEventRecord(e0, st) != cudaSuccess) rc = GPUMPI_ECUDA;
    for (int i = 0; i < reps && !rc; i++) rc = gpumpi_plan_launch(plan, st);
    if (!rc && cudaEventRecord(e1, st) != cudaSuccess) rc = GPUMPI_ECUDA;
    float ms = 0.0f;
    if (!rc && cudaStreamSynchronize(st) != cudaSuccess) rc = GPUMPI_ECUDA;
    if (!rc && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) rc = GPUMPI_ECUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc) rc = gpumpi_api_status(nullptr, 0);
    *us = 1000.0 * ms / reps;
    return rc;
}

}  // namespace

extern "C" int gpumpi_autotune(gpumpi_coll_desc* descs, int ndesc, const gpumpi_tune_opts* opts,
                               int* batched_threads, int* plain_threads, int* plain_algos) {
    if (!descs || ndesc <= 0) return GPUMPI_EINVAL;
    const int reps = opts && opts->reps > 0 ? opts->reps : 5;
    const bool verbose = opts && opts->verbose;
    const char* cache_path = opts ? opts->cache_path : nullptr;
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        set_last_error("gpumpi_autotune: no CUDA device");
        return GPUMPI_ECUDA;
    }
    const std::string gpu = prop.name;
    std::map<std::string, Choice> cache;   // key: shape + ' ' + threads
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line;
        while (std::getline(in, line)) {
            const size_t a = line.find('|'), b = line.rfind('|');
            if (a == std::string::npos || b == a || line.substr(0, a) != gpu) continue;
            Choice c;
            std::istringstream v(line.substr(b + 1));
            if (v >> c.algo >> c.us) cache[line.substr(a + 1, b - a - 1)] = c;
        }
    }
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return GPUMPI_ECUDA;
    std::vector<std::string> fresh;
    int rc = GPUMPI_OK;
    // ---- plain form: best schedule per shape and thread count
    std::vector<std::vector<Choice>> best(ndesc, std::vector<Choice>(kNT));
    for (int i = 0; i < ndesc && !rc; i++) {
        const std::string shape = shape_key(descs[i]);
        for (int ti = 0; ti < kNT && !rc; ti++) {
            const int t = kThreads[ti];
            const std::string key = shape + ' ' + std::to_string(t);
            auto it = cache.find(key);
            if (it == cache.end()) {
                Choice c;
                for (int algo : algos_of(descs[i].op)) {
                    gpumpi_coll_desc d = descs[i];
                    d.algo = algo;
                    gpumpi_plan_t plan = nullptr;
                    const int prc = gpumpi_plan_create(&d, 1, t, 0, &plan);
                    if (prc == GPUMPI_ENORES) break;   // not co-resident at this thread count
                    if (prc) {
                        rc = prc;
                        break;
                    }
                    double us = 0.0;
                    rc = time_plan(plan, reps, st, &us);
                    gpumpi_plan_destroy(plan);
                    if (rc) break;
                    if (verbose)
                        fprintf(stderr, "GPUMPI tune: [%s] algo %d threads %d: %.2f us\n", shape.c_str(), algo, t, us);
                    if (c.us < 0 || us < c.us) {
                        c.algo = algo;
                        c.us = us;
                    }
                }
                if (rc) break;
                it = cache.emplace(key, c).first;
                fresh.push_back(key);
            }
            best[i][ti] = it->second;
        }
    }
    if (!rc) {
        for (int i = 0; i < ndesc; i++) {
            int bt = -1;
            for (int ti = 0; ti < kNT; ti++)
                if (best[i][ti].us >= 0 && (bt < 0 || best[i][ti].us < best[i][bt].us)) bt = ti;
            if (bt < 0) {
                set_last_error("gpumpi_autotune: a descriptor fits at no thread count");
                rc = GPUMPI_ENORES;
                break;
            }
            if (plain_threads) plain_threads[i] = kThreads[bt];
            if (plain_algos) plain_algos[i] = best[i][bt].algo;
        }
    }
    // ---- batched form, measured in the batched launch
    if (!rc && batched_threads) {
        std::vector<gpumpi_coll_desc> work(descs, descs + ndesc);
        for (auto& d : work) d.sync = 0;
        double best_us = -1.0;
        int best_t = -1;
        std::vector<int> best_algo(ndesc), best_sync(ndesc, 0);
        auto time_batched = [&](int t, double* us) -> int {
            gpumpi_plan_t plan = nullptr;
            const int prc = gpumpi_plan_create(work.data(), ndesc, t, 1, &plan);
            if (prc) return prc;
            const int trc = time_plan(plan, reps, st, us);
            gpumpi_plan_destroy(plan);
            return trc;
        };
        for (int ti = 0; ti < kNT && !rc; ti++) {
            for (int i = 0; i < ndesc; i++) work[i].algo = best[i][ti].us >= 0 ? best[i][ti].algo : 0;
            double us = 0.0;
            const int trc = time_batched(kThreads[ti], &us);
            if (trc == GPUMPI_ENORES) continue;
            if (trc) {
                rc = trc;
                break;
            }
            if (verbose) fprintf(stderr, "GPUMPI tune: batched threads %d: %.2f us\n", kThreads[ti], us);
            if (best_us < 0 || us < best_us) {
                best_us = us;
                best_t = ti;
                for (int i = 0; i < ndesc; i++) best_algo[i] = work[i].algo;
            }
        }
        if (!rc && best_t < 0) {
            set_last_error("gpumpi_autotune: the batched list fits at no thread count");
            rc = GPUMPI_ENORES;
        }
        // group refinement at the winning thread count.  Each change is compared
        // against the configuration it would replace, the two timed in
        // alternation (the best of PAIRED_ROUNDS each) and adopted only when
        // faster by more than ADOPT_MARGIN: launches of one configuration
        // differ by about a percent from run to run, more than some of the
        // differences between schedules.
        constexpr int PAIRED_ROUNDS = 3;
        constexpr double ADOPT_MARGIN = 0.005;
        auto time_config = [&](const std::vector<int>& algo, const std::vector<int>& sync, double* us) -> int {
            for (int i = 0; i < ndesc; i++) {
                work[i].algo = algo[i];
                work[i].sync = sync[i];
            }
            return time_batched(kThreads[best_t], us);
        };
        // 1 when (algo, sync) beats the current best; its time in *us
        auto better = [&](const std::vector<int>& algo, const std::vector<int>& sync, double* us, int* out) -> int {
            double cand = 1e300, inc = 1e300;
            for (int r = 0; r < PAIRED_ROUNDS; r++) {
                double t = 0.0;
                int trc = time_config(algo, sync, &t);
                if (trc) return trc;
                cand = std::min(cand, t);
                trc = time_config(best_algo, best_sync, &t);
                if (trc) return trc;
                inc = std::min(inc, t);
            }
            *us = cand;
            *out = cand < inc * (1.0 - ADOPT_MARGIN);
            return 0;
        };
        std::vector<std::pair<int, int>> groups;
        for (int i = 0; i < ndesc && !rc; i++) {
            const std::pair<int, int> g(descs[i].op, descs[i].dtype);
            if (std::find(groups.begin(), groups.end(), g) == groups.end()) groups.push_back(g);
        }
        for (size_t gi = 0; gi < groups.size() && !rc; gi++) {
            auto in_group = [&](int i) {
                return descs[i].op == groups[gi].first && descs[i].dtype == groups[gi].second;
            };
            // candidates: one schedule for every call of the group, then, for each
            // schedule a the group's calls use, those calls moved to schedule b
            // (the plain form's per-call picks are a mix whose parts the batched
            // launch ranks differently)
            const std::vector<int> cands = algos_of(groups[gi].first);
            std::vector<std::pair<int, int>> moves;   // (from, to); from = -1: every call
            for (int b : cands) moves.emplace_back(-1, b);
            for (int a : cands)
                for (int b : cands)
                    if (a != b) moves.emplace_back(a, b);
            for (size_t mi = 0; cands.size() >= 2 && mi < moves.size() && !rc; mi++) {
                std::vector<int> algo(best_algo);
                bool changed = false;
                for (int i = 0; i < ndesc; i++)
                    if (in_group(i) && (moves[mi].first < 0 || algo[i] == moves[mi].first) &&
                        algo[i] != moves[mi].second) {
                        algo[i] = moves[mi].second;
                        changed = true;
                    }
                if (!changed) continue;   // nothing to move, or the current best already
                double us = 0.0;
                int adopt = 0;
                rc = better(algo, best_sync, &us, &adopt);
                if (rc) break;
                if (verbose)
                    fprintf(stderr, "GPUMPI tune: batched group op %d dtype %d algo %d -> %d: %.2f us%s\n",
                            groups[gi].first, groups[gi].second, moves[mi].first, moves[mi].second, us,
                            adopt ? " (adopted)" : "");
                if (adopt) best_algo = algo;
            }
            if (rc) break;
            // the group's calls with flag rounds (a launch-ordered plan leaves its
            // ranks unsynchronised; readers of one buffer that run in step share
            // its lines in L2)
            std::vector<int> sync(best_sync);
            for (int i = 0; i < ndesc; i++)
                if (in_group(i)) sync[i] = 1;
            double us = 0.0;
            int adopt = 0;
            rc = better(best_algo, sync, &us, &adopt);
            if (rc) break;
            if (verbose)
                fprintf(stderr, "GPUMPI tune: batched group op %d dtype %d with flag rounds: %.2f us%s\n",
                        groups[gi].first, groups[gi].second, us, adopt ? " (adopted)" : "");
            if (adopt) best_sync = sync;
        }
        if (!rc) {
            *batched_threads = kThreads[best_t];
            for (int i = 0; i < ndesc; i++) {
                descs[i].algo = best_algo[i];
                descs[i].sync = best_sync[i];
            }
        }
    } else if (!rc) {
        for (int i = 0; i < ndesc; i++) descs[i].algo = plain_algos ? plain_algos[i] : descs[i].algo;
    }
    cudaStreamDestroy(st);
    if (!rc && cache_path && !fresh.empty()) {
        std::ofstream out(cache_path, std::ios::app);
        for (const std::string& k : fresh) {
            const Choice& c = cache[k];
            out << gpu << '|' << k << '|' << c.algo << ' ' << c.us << '\n';
        }
    }
    return rc;
}
