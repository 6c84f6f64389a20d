// workspace.h -- device buffers of one level geometry (the opaque object
// behind pyrsgm_create_workspace).  One cudaMalloc, carved into:
//   featL, featR  uint4  [h][w]     census descriptors (dense words) or BT operands
//   base          int16  [h][w]     refine label base (kNoParent = rejected)
//   C             int16  [h][w][D]  matching cost
//   V             int16  [h][w][D]  aggregation volume
//   Vl, Vr        int16  [h][w][D]  L->R and R->L path sums (16/32/64 labels only)
//   disp_raw      int16  [h][w]     disparity*16 before the median
//   conf_raw      float  [h][w]     confidence before the median reset
//   keys          u32    [h][w]     disp2 candidates (cost << 16 | 0xFFFF - x)
//   lut           int    [256]      adaptive-P2 table
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "sgm_common.cuh"

namespace pg {

struct Workspace {
    int width = 0, height = 0, disp = 0;
    void* mem = nullptr;
    size_t bytes = 0;
    bool owned = false;
    int debug = 0;
    uint4* featL = nullptr;
    uint4* featR = nullptr;
    int16_t* base = nullptr;
    int16_t* C = nullptr;
    int16_t* V = nullptr;
    int16_t* Vl = nullptr;
    int16_t* Vr = nullptr;
    int16_t* disp_raw = nullptr;
    float* conf_raw = nullptr;
    unsigned* keys = nullptr;
    int* lut = nullptr;

    static size_t bytes_for(int w, int h, int D);
    // Lay the buffers of a (w, h, D) geometry out from `p` (bytes_for bytes).
    void carve(unsigned char* p, int w, int h, int D);
    int ensure(int w, int h, int D);
    void release();
};

void sanitize_p2(int& adaptive, float& alpha, float& beta, float& lower, float& upper);
void fill_workspace_ptrs(LevelDesc& d, const Workspace& ws);
int run_level_single(const LevelDesc& d, cudaStream_t st, float alpha, float beta, float lower, float upper,
                     const char* what);

}  // namespace pg
