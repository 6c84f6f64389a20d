// pair_plan.h -- the device resources and level descriptors of one stereo
// pair shape (width, height, validated parameters): what
// StereoMatcher::StereoMatcher allocates in the reference
// (src/stereo_matcher.cpp:164-217), in one arena.  Shared by
// pyrsgm::StereoMatcher and the batch engine.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstddef>
#include <cstdint>

#include "pyrsgm/pyrsgm.h"
#include "sgm_launch.h"
#include "workspace.h"

namespace pyrsgm {
// Level geometry of a validated parameter set, src/stereo_matcher.cpp:169-193.
void levelGeometry(int w, int h, const Params& params, std::array<LevelInfo, 5>& info);
}  // namespace pyrsgm

namespace pg {

struct PairPlan {
    static constexpr int kMaxLevels = 4;

    int width = 0, height = 0;
    pyrsgm::Params params;  // validated
    int levels = 0;
    std::array<pyrsgm::LevelInfo, kMaxLevels + 1> info{};
    void* arena = nullptr;
    size_t arena_bytes = 0;
    std::array<Workspace, kMaxLevels + 1> ws{};
    std::array<uint8_t*, kMaxLevels + 1> pyrL{}, pyrR{};
    std::array<int16_t*, kMaxLevels + 1> disp16{};
    std::array<float*, kMaxLevels + 1> conf{};
    std::array<int, kMaxLevels + 1> pitch8{}, pitch16{}, pitch32{};  // bytes / elements / elements
    float* conf0 = nullptr;
    int* lut = nullptr;
    int adaptive = 0;
    float alpha = 0, beta = 0, lower = 0, upper = 0;

    // Allocates the arena; builds the adaptive-P2 table on `st` (no host sync).
    // Throws std::runtime_error on CUDA failure.
    PairPlan(int w, int h, const pyrsgm::Params& validated, cudaStream_t st = nullptr);
    ~PairPlan();
    PairPlan(const PairPlan&) = delete;
    PairPlan& operator=(const PairPlan&) = delete;

    // Device bytes of a plan of this shape (admission control).
    static size_t bytesFor(int w, int h, const pyrsgm::Params& validated);

    int postFlags(int level) const;
    // Level descriptor with internal buffers; level 0 I/O still unset.
    LevelDesc levelDesc(int level) const;
    // Level 0 descriptor bound to caller images and outputs.  A null conf with
    // a non-null disp32 uses the plan's scratch confidence.
    LevelDesc level0(const uint8_t* L, size_t lp, const uint8_t* R, size_t rp, int16_t* d16, size_t d16p,
                     float* d32, size_t d32p, float* c, size_t cp) const;
    // pyrDown of both views into `level` (1..levels), from caller level 0 or the plan's level-1 images.
    void pyrdownDescs(int level, const uint8_t* L, size_t lp, const uint8_t* R, size_t rp,
                      PyrDownDesc out[2]) const;
};

}  // namespace pg
