// sgm_launch.h -- host-side launch interface of the pyrsgm-gb300 kernels.
//
// Every stage is launched for a batch of independent level jobs (one stereo
// pair's level each); a single-pair call is a batch of one.  Job
// descriptors travel by value in the kernel parameter block, so a launch
// needs no host-to-device copy and can be captured in a CUDA graph.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "check.h"
#include "sgm_common.cuh"

namespace pg {

constexpr int kBatchJobs = 64;  // level jobs per batched launch
constexpr int kBatchPyr = 32;   // pyrDown images per batched launch

struct PyrDownDesc {
    const uint8_t* src;
    uint8_t* dst;
    int sstep, sw, sh, dstep, dw, dh;
};

template <int NB>
struct PyrDownBatch {
    PyrDownDesc d[NB];
    int n;
};

// Largest extents over the jobs of one launch (grid sizing).
struct LevelExtent {
    int max_w = 0, max_h = 0, max_D = 0;
    long long max_vox = 0;
    bool any_refine = false;
};

template <int NJ>
LevelExtent extent_of(const Jobs<NJ>& j)
{
    LevelExtent e;
    for (int i = 0; i < j.n; ++i) {
        const LevelDesc& d = j.d[i];
        e.max_w = std::max(e.max_w, d.w);
        e.max_h = std::max(e.max_h, d.h);
        e.max_D = std::max(e.max_D, d.D);
        e.max_vox = std::max(e.max_vox, (long long)d.w * d.h * d.D);
        e.any_refine = e.any_refine || d.refine;
    }
    return e;
}

// Sums over the jobs of a launch (algorithmic-byte accounting).
template <int NJ>
double jobs_px(const Jobs<NJ>& j)
{
    double s = 0;
    for (int i = 0; i < j.n; ++i) s += (double)j.d[i].w * j.d[i].h;
    return s;
}
template <int NJ>
double jobs_vox(const Jobs<NJ>& j)
{
    double s = 0;
    for (int i = 0; i < j.n; ++i) s += (double)j.d[i].w * j.d[i].h * j.d[i].D;
    return s;
}

// Aggregation kernel variant: G lanes per path chain, K labels per lane,
// G*K >= D (padding labels behave as permanently invalid).
struct PathShape {
    int G, K;
};
PathShape path_shape(int D);
// Kernel family of a label count: 10000 + D for the thread-per-chain packed
// kernels, else G * 100 + K of the lane-parallel ones.  Jobs of one
// aggregation launch share it.
inline int path_variant(int D)
{
    if (uses_packed(D)) return 10000 + D;
    const PathShape s = path_shape(D);
    return s.G * 100 + s.K;
}

// Multiprocessor count of the current device (cached per device).
int sm_count();

// A second stream and two events paired with the main stream `st` (per
// calling thread and device), for launching independent kernels side by
// side (fork: record `fork` on st, `aux` waits; join: record `join` on
// `aux`, st waits).  Under stream capture this becomes two graph branches.
// Null `aux` when they could not be created: run sequentially.
struct ForkStreams {
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
ForkStreams& fork_streams(cudaStream_t st);
// 0 (choose per launch), 8, or 2/4: the packed kernels' words per thread.
int packed_words_override();
// Warps per SM the NW = 8 shape must fill before a launch takes it.
int packed_min_warps_per_sm();
// 1: fused two-pass form of the 16-label pyramid levels (opt-in).
int fused_mode();
// T->B pass with the winner-take-all for those levels: 0 never, 1 when a
// launch fills the GPU (default), 2 always.
int tbw_mode();

// Measuring shape choice for the 16/32/64-label aggregation (opt-in,
// pyrsgm_gb300_set_autotune).  A launch is keyed by its label count, mode,
// total rows and widest level; while the calling thread is in a tuning
// scope (the batch engine's first, uncaptured run of a new batch) a key
// without an entry times both kernel shapes on the launch stream (twice
// each, host-synchronising; the outputs of either are identical) and keeps
// the faster.  Outside a tuning scope a recorded entry is used and an
// unknown key falls back to the rule of packed_nw().
struct TuneKey {
    int D, pyr, rows, w;
    bool operator<(const TuneKey& o) const
    {
        return D != o.D ? D < o.D : pyr != o.pyr ? pyr < o.pyr : rows != o.rows ? rows < o.rows : w < o.w;
    }
};
struct TuneEntry {
    int nw;              // chosen words per thread
    float ms_wide;       // NW = 8 shape, best of two
    float ms_spread;     // spread shape (NW = 2, or 4 for 64 labels), best of two
};
bool autotune_enabled();
bool tuning_thread();
// RAII: marks the calling thread as allowed to measure.
struct TuningScope {
    TuningScope();
    ~TuningScope();
    bool prev;
};
bool tune_lookup(const TuneKey& k, TuneEntry& out);
void tune_store(const TuneKey& k, const TuneEntry& e);

// Count of kernel launches issued by this library (process-wide); a CUDA
// graph replay counts the kernels it contains.
void count_launch();
void count_launches(unsigned long long n);
unsigned long long launch_count();

template <int NB>
cudaError_t launch_pyrdown(const PyrDownBatch<NB>& b, int max_dw, int max_dh, cudaStream_t st);
cudaError_t launch_p2_table(int* lut, int P2, float alpha, float beta, float lower, float upper,
                            cudaStream_t st);
template <int NJ>
cudaError_t launch_prepare(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st);
template <int NJ>
cudaError_t launch_cost(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st);
// All jobs in one call share pyr (mode) and the path shape of their D.
template <int NJ>
cudaError_t launch_paths(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st);
template <int NJ>
cudaError_t launch_post(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st);

}  // namespace pg
