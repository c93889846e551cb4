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
 * sent to each peer. */
typedef struct gpumpi_coll_desc {
    gpumpi_comm_t comm;
    int op;
    int dtype;
    int redop;
    int root;
    uint64_t count;
    void* const* sendbufs;
    void* const* recvbufs;
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
/* Enqueue the plan on a stream (asynchronous). */
int gpumpi_plan_launch(gpumpi_plan_t plan, void* stream);
/* Capture the plan's launches once as a CUDA graph; later launches replay it. */
int gpumpi_plan_capture(gpumpi_plan_t plan, void* stream);
/* Host-buffer form: per-rank host->device copies of the send data, the plan,
 * device->host copies of the results, all enqueued on one stream.  host_send
 * and host_recv list, descriptor by descriptor (creation order), one host
 * pointer per rank; nullptr entries are skipped.  Reports the bytes copied. */
int gpumpi_plan_run_host(gpumpi_plan_t plan, void* const* host_send, void* const* host_recv,
                         void* stream, uint64_t* h2d_bytes, uint64_t* d2h_bytes);
int gpumpi_plan_destroy(gpumpi_plan_t plan);

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

/* Number of kernel launches this process issued through the collective API. */
uint64_t gpumpi_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* GPUMPI_H */
