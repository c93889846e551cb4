// Host-side description of one device MPI job: where each piece of its state
// sits inside one device allocation.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

#include <string>
#include <vector>

#include "gpumpi.h"
#include "rt.cuh"

namespace gm {

struct HostJob {
    char* base = nullptr;        // device allocation
    size_t total = 0;
    size_t zero_off = 0, zero_bytes = 0;   // control state cleared before each launch
    size_t clsp_off = 0, clsp_bytes = 0;   // allocator page lists, filled with 0xff
    size_t job_off = 0;                    // device copy of `job`
    int nranks = 0;
    Job job;                               // host copy with device pointers
    CommShared world;                      // host copies of the communicator headers
    std::vector<CommShared> selfs;
};

void opts_defaults(gpumpi_opts* o);
// Layout of a job of n ranks; fills hj when base is not null.  Returns bytes.
size_t host_job_layout(HostJob& hj, const gpumpi_opts& o, int n, int job_id, char* base);
size_t job_footprint(const gpumpi_opts& o, int n);
int host_job_init(HostJob& hj, cudaStream_t st);
int choose_threads(const void* kernel, int n, int requested, size_t smem, int* max_resident);
// Dynamic shared memory for `need` co-resident rank blocks of `kernel` at T
// threads: BlockCtx plus the largest bulk-copy staging area (64, 32, 16 or
// 8 KiB, or none) that still lets them all be resident.
size_t pick_rank_smem(const void* kernel, int T, int need);
void set_last_error(const char* msg);

// Device image of a program's argv (pointer table + strings, relocated to `dev`).
size_t argv_image_bytes(int argc, char** argv);
void argv_image(int argc, char** argv, char* dev, std::vector<char>& img);

// What a finished job left in its memory, copied back by job_collect.
struct JobResult {
    int status[16];
    std::vector<int> rets;
    std::string out, err, errmsg, diag;
    bool truncated = false;
    int exit_code = 0;
};
int job_collect(HostJob& hj, cudaStream_t st, JobResult& r);
double now_seconds();

}  // namespace gm
