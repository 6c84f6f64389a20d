// profiler.h -- per-kernel event timing hooks (see profiler.cu).
#pragma once

#include <cuda_runtime.h>

namespace pg {

// Kernel kinds reported by pyrsgm_gb300_profile_read.
enum ProfKind {
    PK_PYRDOWN = 0,
    PK_FEATURES = 1,
    PK_LABELS = 2,
    PK_COST = 3,
    PK_PATH_TB = 4,
    PK_PATH_ROW = 5,
    PK_POST = 6,
    PK_P2TABLE = 7,
    PK_WTA = 8,
    PK_TBLR = 9,   // fused T->B + L->R pass (16-label pyramid levels)
    PK_RLW = 10,   // fused R->L + winner-take-all pass
    PK_TBW = 11,   // T->B pass with the winner-take-all folded in
    PK_COUNT
};

bool prof_enabled();
void prof_begin(cudaStream_t st);
void prof_end(int kind, double algorithmic_bytes, cudaStream_t st);

}  // namespace pg
