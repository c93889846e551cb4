// Program entry: the kernel whose thread blocks are the ranks of a converted
// program, and the exported gpumpi_main().  Linked into every program binary
// (it calls the program's __gpu_main, which the runtime library alone lacks).
// Counterpart of __gpu_main_caller and main in gpu_libs/gpu_main/main.cu:103-322.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gpumpi.h"
#include "rt.cuh"

extern __device__ int __gpu_main(int argc, char** argv);
extern __device__ int __gpu_max_threads();

namespace gm {
__device__ bool program_block_begin(const Launch& L);
__device__ void program_block_end(const Launch& L);
}

// The name converted programs use for the start of dynamic shared memory
// (include/gpumpi/global_vars.cuh); it must alias the runtime's block context.
extern __shared__ __align__(16) char __gpumpi_dsmem[];

// Run the rank set up in this block: thread 0 runs the program, the other
// threads execute its MPI calls.  Returns when the rank has finished.
static __device__ void run_rank() {
    using namespace gm;
    BlockCtx& b = bctx();
    if (threadIdx.x == 0) {
        int rc;
        if (b.slot >= __gpu_max_threads()) {
            job_fail(b.job, b.rank, MPI_ERR_INTERN,
                     "rank slots exceed the per-rank global arrays the program was compiled with "
                     "(GPU_MPI_MAX_RANKS)");
            rc = 1;
        } else if ((const void*)__gpumpi_dsmem != (const void*)&b) {
            job_fail(b.job, b.rank, MPI_ERR_INTERN, "per-rank globals cannot find the rank slot");
            rc = 1;
        } else {
            rc = __gpu_main(b.job->argc, b.job->argv);
        }
        cluster_release();
        rank_finish(rc);
        b.call.op = OP_EXIT;
        bar_named(1, b.T);
    } else {
        helper_loop();
    }
}

extern "C" __global__ void __launch_bounds__(1024) gpumpi_program_kernel(gm::Launch L) {
    using namespace gm;
    if (!program_block_begin(L)) {
        program_block_end(L);
        return;
    }
    if (bctx().cl_rank > 0) {   // a helper block of a cluster rank: shares of its parallel loops
        cluster_helper_loop();
        return;
    }
    run_rank();
    program_block_end(L);
}

// Serving runtime (server.cu): blocks 0..nworkers-1 are rank slots that run
// one rank of an admitted job after another; block nworkers is the admin
// block.  A rank that ends with exit() retires its leader thread, and with it
// the block: its slot is reported lost and receives no further ranks.
extern "C" __global__ void __launch_bounds__(1024) gpumpi_server_kernel(gm::ServerArgs A) {
    using namespace gm;
    if ((int)blockIdx.x == A.nworkers) {
        server_admin(A);
        return;
    }
    const int w = (int)blockIdx.x;
    if (threadIdx.x == 0) {
        u32 sm;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(sm));
        A.worker_sm[w] = (int)sm;
        __threadfence();
    }
    u64 seen = 0;
    Job* job;
    int rank, slot;
    while (server_take(A, w, &seen, &job, &rank, &slot)) {
        rank_block_setup(job, rank, A.slot_base + slot);
        run_rank();
        if (threadIdx.x != 0 && *(volatile int*)&bctx().priv->exited) {
            // the leader thread has left the kernel (exit(), abort(), a failed assert)
            if (threadIdx.x == 1) {
                A.lost[slot] = 1;
                __threadfence();
            }
            return;
        }
        __syncthreads();
    }
}

extern "C" int gpumpi_main(int argc, char** argv) {
    for (int i = 1; i < argc; i++) {
        if (strcmp(argv[i], "---gpumpi") != 0) continue;
        for (int k = i + 1; k < argc; k++)
            if (strcmp(argv[k], "--serve") == 0) {
                return gpumpi_serve_main((const void*)gpumpi_server_kernel, argc, argv);
            }
        break;
    }
    gpumpi_opts o;
    int pos = gpumpi_parse_args(argc, argv, &o);
    if (pos == -1) {
        fprintf(stderr, "You should specify gpumpi related options after '---gpumpi'\n");
        return 1;
    }
    if (pos < 0) return 1;
    return gpumpi_run_program((const void*)gpumpi_program_kernel, pos, argv, &o);
}
