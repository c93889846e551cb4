/*
 * C ABI of the GB300 device MPI runtime.
 *
 * Two groups of entry points:
 *
 *  1. Program launcher.  A converted MPI program (converter output compiled
 *     against include/gpumpi/*.h.cuh) is linked with the runtime into an
 *     executable or shared library that exports gpumpi_main().  It replaces
 *     the reference's host `main` in gpu_libs/gpu_main/main.cu:134-322 and keeps
 *     its command line: program arguments, then a literal "---gpumpi",
 *     then launcher options -n -g -b -s -p -e (main.cu:49-98).
 *
 *  2. Host-driven collectives on device buffers, one call per collective
 *     ("plain": one kernel launch per call) or many communicators and calls
 *     in one persistent launch ("batched"), optionally captured as a CUDA
 *     graph.  These have no counterpart in the reference, which only offered
 *     the device-side MPI_* calls; they expose the same device schedules
 *     (mpi.cu:77-408 in the reference) to host code.
 *
 * All pointers are plain device or host addresses; streams are cudaStream_t
 * passed as void*.  Every function returns 0 on success or a nonzero
 * GPUMPI_E* / MPI error code.
 */
#ifndef GPUMPI_H
#define GPUMPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- error codes of the host API ---- */
#define GPUMPI_OK 0
#define GPUMPI_EINVAL 1001      /* bad argument */
#define GPUMPI_ECUDA 1002       /* a CUDA runtime call failed */
#define GPUMPI_ENORES 1003      /* ranks cannot all be resident on the GPU at once */
#define GPUMPI_EJOB 1004        /* the device job reported an error (see gpumpi_last_error) */
#define GPUMPI_EAGAIN 1005      /* gpumpi_poll: the job has not finished yet */

/* ---- launcher (section 1) ---- */

/* Launcher options; zero fields take defaults. */
typedef struct gpumpi_opts {
    int nranks;              /* -n: MPI ranks (default: blocks * threads, as -g/-b in the reference) */
    int threads_per_rank;    /* -t: threads in each rank block (0 = choose) */
    size_t stack_bytes;      /* -s: per-thread stack limit (default 16 KiB) */
    size_t heap_bytes;       /* -p: device heap for malloc (default 1 GiB) */
    int max_requests;        /* -e: outstanding requests per rank (default 1024) */
    size_t eager_bytes;      /* eager/rendezvous threshold (default 4096) */
    double timeout_s;        /* bound on every device wait (default 60 s) */
    size_t out_bytes;        /* stdout and stderr buffer size per job (default 16 MiB) */
    double max_seconds;      /* host wall-clock limit of the whole run, 0 = none */
    int verbose;             /* print GPUMPI: launch lines on stderr */
    int blocks_per_rank;     /* --blocks-per-rank: each rank a cluster of this many thread
                                blocks (1, 2, 4, 8; 0 = 1); parallel loops span all of them */
    int one_cluster;         /* --one-cluster: all ranks (at most 16) in one thread-block
                                cluster, mailboxes in distributed shared memory */
} gpumpi_opts;

/* Exported by every program library: parse "---gpumpi" options from argv,
 * run the program's ranks on the GPU, print their output, return the exit
 * status (0 when every rank returned 0 and no rank failed).
 * Replaces: gpu_libs/gpu_main/main.cu:134-322 (host main). */
int gpumpi_main(int argc, char** argv);

/* Parse the options after "---gpumpi" (main.cu:49-98).  Returns the index of
 * "---gpumpi" in argv (the program's argc), or -1 when it is missing. */
int gpumpi_parse_args(int argc, char** argv, gpumpi_opts* opts);

/* Run a program kernel (the library-internal entry that calls __gpu_main)
 * with explicit options.  prog_argc/prog_argv are passed to __gpu_main.
 * Replaces: the launch and poll sequence of main.cu:163-321. */
int gpumpi_run_program(const void* program_kernel, int prog_argc, char** prog_argv,
                       const gpumpi_opts* opts);

/* Text of the last device job error of this process. */
const char* gpumpi_last_error(void);

/* ---- serving: many jobs of one program, admitted by HBM footprint ---- */

/* One job: program arguments (argv[0] first), ranks, device heap, arrival. */
typedef struct gpumpi_job_spec {
    int argc;
    char** argv;
    int nranks;
    size_t heap_bytes;       /* 0 = 256 MiB */
    double submit_s;         /* arrival, seconds after serving starts */
} gpumpi_job_spec;

typedef struct gpumpi_serve_opts {
    size_t pool_bytes;       /* HBM reserved for the memory of admitted jobs (0 = half of free memory) */
    int max_slots;           /* rank blocks that may run at once (0 = what the GPU holds, at most 1024) */
    int threads_per_rank;    /* 0 = 128 */
    double timeout_s;        /* bound on every device wait (0 = 60 s) */
    double max_seconds;      /* wall-clock limit of the whole run (0 = none) */
    int verbose;
} gpumpi_serve_opts;

typedef struct gpumpi_job_result {
    int exit_code;           /* 0 when every rank returned 0 and nothing failed */
    int error;               /* first device error code of the job (0 = none) */
    size_t footprint;        /* bytes of the HBM pool the job held */
    int slot_base;           /* first rank slot of the job (-1 = never admitted) */
    double submit_s, start_s, end_s;   /* seconds after serving started */
    char* out;               /* the job's stdout text; release with gpumpi_free */
    char* err;               /* its stderr text and launcher diagnostics; gpumpi_free */
} gpumpi_job_result;

/* Run every job to completion on a server (below): each job is submitted at
 * its arrival time and admitted once its job memory fits in a free range of
 * the pool and a contiguous range of idle rank slots is free.  server_kernel
 * is the program's gpumpi_server_kernel.  No counterpart in the reference,
 * which ran one program per process (gpu_libs/gpu_main/main.cu:163-321).
 * Returns 0, GPUMPI_EJOB when a job failed (see its result), or an error code. */
int gpumpi_serve(const void* server_kernel, const gpumpi_job_spec* jobs, int njobs,
                 const gpumpi_serve_opts* opts, gpumpi_job_result* results);

/* Online serving.  gpumpi_server_start launches server_kernel (the program's
 * gpumpi_server_kernel) once, as one persistent cooperative launch of worker
 * blocks (rank slots) and an admin block, and starts a host thread that
 * admits submitted jobs as their HBM footprint and rank slots free up; jobs
 * run side by side, and a finished job's slots and memory go to the next.
 * The admission and completion records travel through a ring in pinned host
 * memory.  No counterpart in the reference, which ran one program per
 * process (gpu_libs/gpu_main/main.cu:163-321) and whose device->host queue
 * went unused (gpu_libs/gpu_libc/cuda_mpi.cuh:392-435). */
typedef struct gpumpi_server_s* gpumpi_server_t;
int gpumpi_server_start(const void* server_kernel, const gpumpi_serve_opts* opts, gpumpi_server_t* server);
/* Queue a job (its argv strings are copied); returns at once with its id.
 * submit_s is ignored: the job arrives now.  Safe to call from any thread. */
int gpumpi_submit(gpumpi_server_t server, const gpumpi_job_spec* job, long long* job_id);
/* The result of a job: waits up to wait_ms (-1: until it has finished, 0:
 * not at all).  Returns 0 and fills *result (times in seconds since the
 * server started; release the texts with gpumpi_free), or GPUMPI_EAGAIN while
 * the job runs or waits.  Each result is returned once. */
int gpumpi_poll(gpumpi_server_t server, long long job_id, int wait_ms, gpumpi_job_result* result);
/* Wait until every submitted job has finished, end the persistent launch and
 * release the server (results not polled are discarded). */
int gpumpi_server_stop(gpumpi_server_t server);

/* Command-line form, used by gpumpi_main when "--serve JOBFILE" follows
 * "---gpumpi": one job per line, "<ranks> <arrival-ms> [arguments...]";
 * "--serve -" reads such lines from standard input and submits each job the
 * moment its line arrives (the arrival time is then ignored), printing each
 * job's output as it finishes.  program_kernel is the program's
 * gpumpi_server_kernel. */
int gpumpi_serve_main(const void* program_kernel, int argc, char** argv);

/* Release memory returned by the runtime (gpumpi_job_result texts). */
void gpumpi_free(void* p);

/* ---- host-driven collectives (section 2) ---- */

typedef struct gpumpi_comm_s* gpumpi_comm_t;

/* Collective kinds of gpumpi_coll_desc.op */
#define GPUMPI_COLL_BARRIER 0
#define GPUMPI_COLL_BCAST 1
#define GPUMPI_COLL_REDUCE 2
#define GPUMPI_COLL_ALLREDUCE 3
#define GPUMPI_COLL_ALLTOALL 4
#define GPUMPI_COLL_ALLGATHER 5

/* Reduction operators (same order as the device MPI_Op handles) */
#define GPUMPI_OP_MAX 0
#define GPUMPI_OP_MIN 1
#define GPUMPI_OP_SUM 2
#define GPUMPI_OP_PROD 3

/* Element types (values of the device MPI_Datatype enum) */
#define GPUMPI_DT_BYTE 29
#define GPUMPI_DT_INT 2
#define GPUMPI_DT_INT64 20
#define GPUMPI_DT_FLOAT 12
#define GPUMPI_DT_DOUBLE 13

/* One collective call over one communicator.  sendbufs/recvbufs are host
 * arrays of nranks device pointers (rank r's buffers).  count is elements per
 * rank: the broadcast length, the reduction length, or for ALLTOALL the block
 * sent to each peer.  algo selects the schedule (0 = by message size):
 *   BCAST      1 every rank copies from the root, 2 binomial tree (log2 P
 *              rounds, each rank copies from its parent once the parent has
 *              its copy; always with flag rounds)
 *   REDUCE     1 root folds all inputs, 2 every rank folds a segment
 *   ALLREDUCE  1 every rank folds all inputs, 2 reduce-scatter + allgather,
 *              3 every rank folds its segment and writes it to every rank
 *   ALLTOALL, ALLGATHER  1 peer blocks one after another by the whole rank
 *              block, 2 one peer block per warp, 3 all peer blocks through
 *              one bulk asynchronous copy pipeline (cp.async.bulk), 4 the
 *              16-byte vectors of all peer blocks spread over every thread
 *              (launch-ordered plans; elsewhere as 0)
 * gpumpi_autotune fills it in, and `sync` in the batched form. */
typedef struct gpumpi_coll_desc {
    gpumpi_comm_t comm;
    int op;
    int dtype;
    int redop;
    int root;
    uint64_t count;
    void* const* sendbufs;
    void* const* recvbufs;
    int algo;
    int sync;    /* 1: this call synchronises its ranks with flag rounds even in a
                    launch-ordered plan (gpumpi_plan_set_sync); 0: the plan's form */
} gpumpi_coll_desc;

/* Create a communicator of nranks rank blocks with its synchronisation state in HBM. */
int gpumpi_comm_create(int nranks, gpumpi_comm_t* comm);
int gpumpi_comm_destroy(gpumpi_comm_t comm);
int gpumpi_comm_size(gpumpi_comm_t comm, int* nranks);

/* Plain form: one cooperative kernel launch of comm-size blocks per
 * descriptor; synchronises the stream and reports device errors. */
int gpumpi_coll_plain(const gpumpi_coll_desc* descs, int ndesc, int threads_per_rank, void* stream);

/* Batched form: every descriptor in one persistent cooperative launch; the
 * blocks of each communicator run that communicator's calls in order.
 * Synchronises the stream and reports device errors. */
int gpumpi_coll_batched(const gpumpi_coll_desc* descs, int ndesc, int threads_per_rank, void* stream);

/* Reusable plan of collective calls (descriptors are copied to the device
 * once).  batched = 0: one launch per descriptor; 1: one launch in total.
 * threads_per_rank 0 = 128. */
typedef struct gpumpi_plan_s* gpumpi_plan_t;
int gpumpi_plan_create(const gpumpi_coll_desc* descs, int ndesc, int threads_per_rank, int batched,
                       gpumpi_plan_t* plan);
/* As gpumpi_plan_create; plain_threads (may be NULL) gives the threads per
 * rank of each descriptor's own launch in the plain form. */
int gpumpi_plan_create_ex(const gpumpi_coll_desc* descs, int ndesc, int threads_per_rank, int batched,
                          const int* plain_threads, gpumpi_plan_t* plan);
/* Enqueue the plan on a stream (asynchronous). */
int gpumpi_plan_launch(gpumpi_plan_t plan, void* stream);
/* Synchronisation of a plan's calls.  mode 0 (the default): when no call of
 * the plan writes memory that another call reads or writes and none is a
 * barrier (checked at creation), the batched launch runs every call in its
 * launch-ordered form, which needs no flag round between the ranks: the
 * inputs were complete when the launch started and the end of the launch
 * orders the results.  A plain launch holds one call and is always
 * launch-ordered in mode 0.  mode 1: every call synchronises its ranks with
 * arrive/depart flags, as the device MPI_* calls do.  Drops a captured graph
 * (capture again to replay).  No counterpart in the reference. */
int gpumpi_plan_set_sync(gpumpi_plan_t plan, int mode);
/* 1 when the plan's launches run the launch-ordered forms, else 0. */
int gpumpi_plan_launch_ordered(gpumpi_plan_t plan);
/* Capture the plan's launches once as a CUDA graph; later launches replay it
 * on the stream given to gpumpi_plan_launch.  `stream` is not used (the
 * capture runs on a private stream). */
int gpumpi_plan_capture(gpumpi_plan_t plan, void* stream);
/* Host-buffer form: per-rank host->device copies of the send data, the plan,
 * device->host copies of the results, all enqueued on one stream.  host_send
 * and host_recv list, descriptor by descriptor (creation order), one host
 * pointer per rank; nullptr entries are skipped.  Reports the bytes copied. */
int gpumpi_plan_run_host(gpumpi_plan_t plan, void* const* host_send, void* const* host_recv,
                         void* stream, uint64_t* h2d_bytes, uint64_t* d2h_bytes);
int gpumpi_plan_destroy(gpumpi_plan_t plan);

/* Autotuner, on the descriptors' own buffers (their contents are
 * overwritten).  Plain form: times every candidate schedule (algo) at every
 * co-resident thread count of each descriptor alone and returns the fastest
 * in plain_algos[i] and plain_threads[i] (either may be NULL).  Batched form
 * (when batched_threads is not NULL): measured in the batched launch itself
 * at every co-resident thread count, then per (collective, type) group; the
 * choice goes to descs[i].algo and *batched_threads (without it,
 * descs[i].algo gets the plain choice).  Plain results are cached in
 * cache_path (one line per shape, thread count and GPU; NULL = no cache).
 * No counterpart in the reference, whose collectives had one schedule each. */
typedef struct gpumpi_tune_opts {
    int reps;                /* timed launches per candidate (0 = 5) */
    const char* cache_path;
    int verbose;
} gpumpi_tune_opts;
int gpumpi_autotune(gpumpi_coll_desc* descs, int ndesc, const gpumpi_tune_opts* opts, int* batched_threads,
                    int* plain_threads, int* plain_algos);

/* Error state of the collective API's device job (a timed-out wait, ...);
 * returns GPUMPI_EJOB and clears it when an error was recorded. */
int gpumpi_api_status(char* msg, int len);

/* Allreduce over nranks device buffers that allocates no device memory.
 * No counterpart in the reference (it had no host-side collective API).
 * For callers that may not allocate on their call path -- a server that
 * reserved all of HBM at start-up, code under a fixed pooled-allocator
 * budget, or a thread that must not let cudaMalloc/cudaFree synchronise the
 * device.  The runtime's synchronisation state lives in a fixed 64 KiB array
 * in device memory, so nranks is limited to 256 (larger requests fail with
 * GPUMPI_EINVAL).  sendbufs/recvbufs are host arrays of nranks device
 * pointers; count elements of dtype are reduced with redop in rank order.
 * The first call on a device looks up the array's address (with that device
 * current) and should therefore come before any stream capture.  All calls
 * share the array: calls whose kernels overlap on the GPU race.  The call
 * synchronises `stream` and returns 0 or an error code. */
int gpumpi_allreduce_noalloc(void* const* sendbufs, void* const* recvbufs, int nranks,
                             uint64_t count, int dtype, int redop, int threads_per_rank,
                             void* stream);

/* ---- allocator churn ---- */

/* Result of gpumpi_malloc_churn. */
typedef struct gpumpi_churn_stats {
    uint64_t allocs;              /* malloc calls */
    uint64_t frees;               /* free calls */
    uint64_t failed;              /* malloc calls that returned NULL */
    uint64_t corrupt;             /* objects whose pattern did not survive until free */
    uint64_t misaligned;          /* pointers not 16-byte aligned */
    double seconds;               /* kernel time (CUDA events) */
    double ops_per_s;             /* (allocs + frees) / seconds */
    uint64_t malloc_cycles_p50;   /* malloc latency percentiles in SM cycles */
    uint64_t malloc_cycles_p99;   /*   (lower edge of a quarter-octave bucket) */
    uint64_t fresh_pages;         /* slab allocator: 64 KiB pages taken from the bump pointer */
    uint64_t partial_pops;        /*   pages taken from the free-chunk stacks */
    uint64_t partial_full;        /*   of those, pages that were full again */
    uint64_t malloc_cycles_mean;  /* mean malloc latency (SM cycles, exact) */
    uint64_t free_cycles_p50;     /* free latency percentiles (bucket lower edges) */
    uint64_t free_cycles_p99;
    uint64_t free_cycles_mean;    /* mean free latency */
} gpumpi_churn_stats;

/* Every thread of a blocks x threads grid runs `iters` rounds of: malloc of
 * floor(2^U) bytes, U uniform in [4, 12); write a pattern over the object; keep
 * at most `live` objects (1..16), verifying and freeing the oldest first.
 * cuda_heap = 0 uses the runtime's slab allocator on a fresh heap of
 * heap_bytes (0 = 4 GiB); cuda_heap = 1 uses CUDA's device malloc/free, the
 * allocator behind the reference's __gpu_malloc (gpu_libs/gpu_libc/stdlib.cu:70-91).
 * Allocates and frees its own device memory; synchronises `stream`. */
int gpumpi_malloc_churn(int blocks, int threads, int iters, int live, uint64_t seed, size_t heap_bytes,
                        int cuda_heap, void* stream, gpumpi_churn_stats* out);

/* The reference's allocator benchmark shape (dynamic_allocator/
 * benchmarks_template.cu:68-202): every thread of a blocks x threads grid
 * allocates one object of `bytes` bytes, writes and checks it, and frees it;
 * the latency of every malloc and free is recorded (mean and percentiles in
 * `out`; allocs/frees/failed/corrupt as in gpumpi_malloc_churn).  cuda_heap
 * as there.  Allocates and frees its own device memory; synchronises `stream`. */
int gpumpi_malloc_bench(int blocks, int threads, size_t bytes, size_t heap_bytes, int cuda_heap, void* stream,
                        gpumpi_churn_stats* out);

/* Number of kernel launches this process issued through the collective API. */
uint64_t gpumpi_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* GPUMPI_H */
