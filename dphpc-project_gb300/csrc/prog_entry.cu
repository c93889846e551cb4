// Program entry: the kernel whose thread blocks are the ranks of a converted
// program, and the exported gpumpi_main().  Linked into every program binary
// (it calls the program's __gpu_main, which the runtime library alone lacks).
// Counterpart of __gpu_main_caller and main in gpu_libs/gpu_main/main.cu:103-322.
#include <stdio.h>

#include "gpumpi.h"
#include "rt.cuh"

extern __device__ int __gpu_main(int argc, char** argv);
extern __device__ int __gpu_max_threads();

namespace gm {
__device__ bool program_block_begin(const Launch& L);
}

extern "C" __global__ void __launch_bounds__(1024) gpumpi_program_kernel(gm::Launch L) {
    using namespace gm;
    if (!program_block_begin(L)) return;
    BlockCtx& b = bctx();
    if (threadIdx.x == 0) {
        int rc;
        if ((int)gridDim.x > __gpu_max_threads()) {
            job_fail(b.job, b.rank, MPI_ERR_INTERN,
                     "grid exceeds the per-rank global arrays the program was compiled with "
                     "(GPU_MPI_MAX_RANKS)");
            rc = 1;
        } else {
            rc = __gpu_main(b.job->argc, b.job->argv);
        }
        rank_finish(rc);
        b.call.op = OP_EXIT;
        bar_named(1, b.T);
    } else {
        helper_loop();
    }
}

extern "C" int gpumpi_main(int argc, char** argv) {
    gpumpi_opts o;
    int pos = gpumpi_parse_args(argc, argv, &o);
    if (pos == -1) {
        fprintf(stderr, "You should specify gpumpi related options after '---gpumpi'\n");
        return 1;
    }
    if (pos < 0) return 1;
    return gpumpi_run_program((const void*)gpumpi_program_kernel, pos, argv, &o);
}
