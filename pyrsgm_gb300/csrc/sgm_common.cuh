// sgm_common.cuh -- level descriptors and device helpers shared by every
// pyrsgm-gb300 kernel.
//
// Layout in HBM (one level of one stereo pair):
//   images            u8, caller-pitched (bytes)
//   features          16 bytes per pixel and view: the census descriptor
//                     (one word per pixel, dense) for the Census cost, or
//                     the Birchfield-Tomasi operands (value + 256, value,
//                     lo + 256, hi; gradient and intensity as 16-bit pairs)
//   label base        int16 per pixel (refine levels); kNoParent marks pixels
//                     whose parent was rejected (no valid label)
//   cost volume C     int16 [y][x][D], d innermost
//   aggregation V     int16 [y][x][D]: top->bottom path costs, then (other
//                     label counts) the partial sums of whichever
//                     horizontal path reaches a pixel first; final totals in
//                     debug mode
//   Vl, Vr            int16 [y][x][D]: L->R and R->L path costs of the
//                     16/32/64-label levels (summed by the WTA kernel)
//   disp_raw/conf_raw int16 / float per pixel (pitch = width)
#pragma once

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

namespace pg {

constexpr int kMax = SHRT_MAX;           // saturation point and invalid-label sentinel
constexpr int16_t kNoParent = INT16_MIN; // label base of a pixel with no valid parent
enum { COST_BT = 0, COST_CENSUS = 1 };
enum { POST_LRCHECK = 1, POST_MEDIAN = 2 };

struct LevelDesc {
    // inputs (device)
    const uint8_t* left;
    const uint8_t* right;
    const int16_t* pdisp;
    const float* pconf;
    // workspace (device)
    uint4* featL;
    uint4* featR;
    int16_t* base;
    int16_t* C;
    int16_t* V;
    int16_t* Vl;      // L->R path sums (packed levels)
    int16_t* Vr;      // R->L path sums (packed levels)
    int16_t* disp_raw;
    float* conf_raw;
    unsigned* keys;   // disp2 candidates: (cost << 16 | 0xFFFF - x) per right-image pixel
    const int* p2lut;
    // outputs (device, optional)
    int16_t* out16;
    float* out32;
    float* outc;
    // pitches: images in bytes, everything else in elements
    int lstep, rstep, pd_pitch, pc_pitch, out16_pitch, out32_pitch, outc_pitch;
    // geometry
    int w, h, pw, ph;
    int D, minD, maxD;
    // mode and parameters
    int pyr;      // 0: single-scale semantics, 1: pyramid level semantics
    int refine;   // pyramid refinement level (labels relative to the parent)
    int cost;     // COST_BT / COST_CENSUS
    int bs, pfc;
    int P1, P2, uniq, maxdiff, post, paths, adaptive;
    float minConf;
    int conf_only_copy;  // pyramid: copy conf when disp32 is not requested
    int debug_acc;       // write the final aggregated volume into V
};

template <int NJ>
struct Jobs {
    LevelDesc d[NJ];
    int n;
};

// Label counts aggregated by the thread-per-chain packed kernels
// (k_paths_packed.cuh); their LR check runs in the post kernel.
__host__ __device__ __forceinline__ bool uses_packed(int D) { return D == 16 || D == 32 || D == 64; }

__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ int iclamp(int v, int lo, int hi) { return imin(imax(v, lo), hi); }
__device__ __forceinline__ int sat16(int v) { return imin(kMax, imax(SHRT_MIN, v)); }

// Geometry-valid local labels of pixel x at a pyramid level: the labels whose
// real disparity base+d lies in [minD, maxD] and projects inside the right
// image (x - (base+d) in [0, w)).  Returns lo > hi when there is none.
__device__ __forceinline__ void label_range(const LevelDesc& J, int x, int base, int& lo, int& hi)
{
    if (base == kNoParent) { lo = 1; hi = 0; return; }
    const int first = imax(J.minD, x - (J.w - 1));
    const int last = imin(J.maxD, x);
    lo = imax(0, first - base);
    hi = imin(J.D - 1, last - base);
}

}  // namespace pg
