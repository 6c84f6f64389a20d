/**
 * @file pyrsgm.h
 * @brief pyrsgm-gb300 C++ API: coarse-to-fine Semi-Global Matching on GB300.
 *
 * Drop-in for the reference C++ API (reference include/pyrsgm/pyrsgm.h:27-146):
 * same namespace, types, defaults, member functions and exceptions.
 *
 *   pyrsgm::Params p;
 *   p.num_disparities = 256;
 *   p.pyramid_levels  = 2;
 *   pyrsgm::StereoMatcher sgm(width, height, p);
 *   sgm.compute(d_left, lp, d_right, rp, d_disp16, dp, nullptr, 0, nullptr, 0, stream);
 */
#pragma once

#include <cstddef>
#include <cstdint>
#include <memory>

#include <cuda_runtime.h>

namespace pyrsgm {

/// Matching cost (reference include/pyrsgm/pyrsgm.h:27-30).
enum class CostMode {
    BirchfieldTomasi = 0,  ///< BT on gradient + intensity, block_size^2 SAD window
    Census = 1             ///< 5x5 Census + Hamming distance
};

/// Matcher parameters; defaults as in reference include/pyrsgm/pyrsgm.h:32-82.
struct Params {
    int num_disparities = 128;   ///< full-resolution range, aligned up to 16, <= 1024
    int min_disparity = 0;       ///< pyramid mode requires 0
    int block_size = 5;          ///< BT SAD window (odd, >= 3); levels >= 2 use 3
    CostMode cost_mode = CostMode::BirchfieldTomasi;
    int p1 = 300;
    int p2 = 2400;
    int uniqueness_ratio = 10;   ///< percent; 0 disables
    int disp12_max_diff = 1;
    bool lr_check = true;
    bool median_filter = true;   ///< 3x3 median on the final level
    int num_paths = 3;           ///< 3 = L->R, T->B, R->L; 2 drops T->B; 1 keeps R->L
    int pre_filter_cap = 63;

    int pyramid_levels = 0;      ///< 0 = single scale; 1..4 = coarse search at 1/2^L
    int pyramid_coarse_disparities = 128;
    int pyramid_max_disparity = 0;   ///< <= 0 selects num_disparities - 1
    float pyramid_min_confidence = 0.05f;

    bool adaptive_p2 = false;
    float p2_alpha = 3.041f;
    float p2_beta = 16.137f;
    float p2_lower_mult = 0.601f;
    float p2_upper_mult = 1.77f;
};

/// Resolve derived values; throws std::invalid_argument for unsupported
/// combinations (reference src/stereo_matcher.cpp:100-148).
Params validateParams(const Params& params);

/// Fixed-point invalid marker of the int16 output.
inline int16_t invalidDisparity16(const Params& params)
{
    return static_cast<int16_t>((params.min_disparity - 1) * 16);
}

/// Per-level geometry (reference include/pyrsgm/pyrsgm.h:95-103).
struct LevelInfo {
    int level = 0;
    int width = 0;
    int height = 0;
    int num_labels = 0;
    int max_disparity = 0;
    int block_size = 0;
    bool refine = false;
};

/**
 * Stereo matcher for a fixed image size.  All device memory is allocated in
 * the constructor (one arena); compute() allocates nothing and is fully
 * asynchronous on the given stream.  Inputs: 8-bit rectified grayscale
 * device images.  Outputs (optional, nullptr to skip): disp16 (disparity*16,
 * invalid = invalidDisparity16()), disp32 (pixels, invalid = 0), conf
 * ([0,1], 0 where invalid).  Replaces reference include/pyrsgm/pyrsgm.h:116-144.
 */
class StereoMatcher {
public:
    StereoMatcher(int width, int height, const Params& params);
    ~StereoMatcher();
    StereoMatcher(StereoMatcher&&) noexcept;
    StereoMatcher& operator=(StereoMatcher&&) noexcept;
    StereoMatcher(const StereoMatcher&) = delete;
    StereoMatcher& operator=(const StereoMatcher&) = delete;

    void compute(const uint8_t* d_left, size_t left_pitch,
                 const uint8_t* d_right, size_t right_pitch,
                 int16_t* d_disp16, size_t disp16_pitch,
                 float* d_disp32, size_t disp32_pitch,
                 float* d_conf, size_t conf_pitch,
                 cudaStream_t stream = nullptr);

    int width() const;
    int height() const;
    const Params& params() const;
    int numLevels() const;
    LevelInfo levelInfo(int level) const;
    size_t deviceMemoryBytes() const;

private:
    struct Impl;
    std::unique_ptr<Impl> impl_;
};

const char* version();

}  // namespace pyrsgm
