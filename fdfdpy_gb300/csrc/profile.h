// Per-kernel-class launch counters and (optional) CUDA-event timing.
// Counting is always on; event timing only between fdfd_profile_enable(1)
// and fdfd_profile_read().  Single-threaded use per process.
#pragma once

#include <cuda_runtime.h>

namespace fdfd {

enum ProfClass {
    PROF_ASSEMBLE = 0,
    PROF_EXTEND_ADD = 1,
    PROF_LU_DIAG = 2,
    PROF_TRSM = 3,
    PROF_SCHUR = 4,
    PROF_SOLVE_FWD = 5,
    PROF_SOLVE_BWD = 6,
    PROF_OTHER = 7,
    PROF_SCHUR_SIMT = 8,
    PROF_NCLASS = 9
};

void prof_begin(int cls, cudaStream_t st);
void prof_end(int cls, cudaStream_t st, int launches);
// Whether event timing is on (graph replays are not timed per class), the
// launch counter of a class, and a count added for the launches of a
// replayed graph.
bool prof_enabled();
long long prof_launches(int cls);
void prof_count(int cls, long long launches);

}  // namespace fdfd
