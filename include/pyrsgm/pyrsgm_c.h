/*
 * pyrsgm_c.h -- C API of pyrsgm-gb300 (coarse-to-fine Semi-Global Matching
 * for NVIDIA GB300 / sm_103a).
 *
 * Drop-in for the reference C API: same functions, argument order, types,
 * constants, ownership and return convention as the reference header
 * include/pyrsgm/pyrsgm_c.h:25-140.  Each declaration below names the
 * reference declaration it replaces.
 *
 *   - Image pointers are DEVICE pointers; pitches ("step") are in bytes.
 *   - Calls only enqueue work on `stream` (no host synchronisation) and return
 *     0 on success, -1 on a bad argument, an allocation failure or a launch
 *     error.  Asynchronous faults surface through cudaGetLastError() /
 *     cudaStreamSynchronize().
 *   - int16 disparity = disparity * 16; invalid = (minDisparity - 1) * 16.
 */
#ifndef PYRSGM_C_H
#define PYRSGM_C_H

#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* costMode (reference include/pyrsgm/pyrsgm_c.h:25-27) */
#define PYRSGM_COST_BT       0   /* Birchfield-Tomasi on gradient + intensity, SAD window */
#define PYRSGM_COST_CENSUS   1   /* 5x5 Census transform + Hamming distance              */

/* postFlags bits (reference include/pyrsgm/pyrsgm_c.h:29-31) */
#define PYRSGM_POST_LRCHECK  1   /* left-right consistency check */
#define PYRSGM_POST_MEDIAN   2   /* 3x3 median of the final disparity */

/*
 * Workspace: device buffers for one (width, height, numDisparities)
 * geometry, re-allocated lazily when the geometry changes.  One workspace per
 * pyramid level and per concurrently running stream.
 * Replaces reference include/pyrsgm/pyrsgm_c.h:38-39.
 */
void* pyrsgm_create_workspace(void);
void  pyrsgm_destroy_workspace(void* workspace);

/*
 * Allocate the workspace for a geometry up front (optional; the compute
 * functions do it on demand).  numDisparities: multiple of 16, <= 1024.
 * Replaces reference include/pyrsgm/pyrsgm_c.h:46.
 */
int pyrsgm_workspace_reserve(void* workspace, int width, int height, int numDisparities);

/*
 * Full-resolution single-scale 3-path SGM.
 * d_disp (int16) may be NULL; d_disp_float and d_conf_float are written only
 * when both are non-NULL.  numPaths 1..3 (3 = left->right, top->bottom,
 * right->left; 2 drops top->bottom; 1 keeps right->left).  adaptiveP2 != 0:
 * P2' = P2 * (lower + (1+alpha-lower) * exp(-|dI|/beta)), clamped to
 * [max(1, P2*lower), P2*upper].
 * Replaces reference include/pyrsgm/pyrsgm_c.h:63-86.
 */
int pyrsgm_compute_single_scale(
    void* workspace,
    const unsigned char* d_left_gray,
    const unsigned char* d_right_gray,
    short* d_disp,
    float* d_disp_float,
    float* d_conf_float,
    size_t left_step_bytes,
    size_t right_step_bytes,
    size_t disp_step_bytes,
    size_t disp_float_step_bytes,
    size_t conf_float_step_bytes,
    int width, int height,
    int numDisparities, int minDisparity,
    int blockSize, int P1, int P2,
    int uniquenessRatio, int disp12MaxDiff,
    int preFilterCap,
    int costMode,
    int postFlags,
    int numPaths,
    int adaptiveP2,
    float p2Alpha, float p2Beta, float p2LowerMult, float p2UpperMult,
    cudaStream_t stream);

/*
 * One pyramid level.
 * refineLevel == 0: search [minDisparity, minDisparity + numDisparities),
 *   capped by maxDisparity; parent inputs are ignored.
 * refineLevel != 0: numDisparities (16; <= 256 accepted) contiguous local
 *   labels around the 2x up-scaled parent disparity; parent pixels that are
 *   invalid or below minConfidence stay invalid.
 * Intermediate levels should pass postFlags = PYRSGM_POST_LRCHECK.
 * Replaces reference include/pyrsgm/pyrsgm_c.h:101-129.
 */
int pyrsgm_compute_level(
    void* workspace,
    const unsigned char* d_left_gray,
    const unsigned char* d_right_gray,
    const short* d_parent_disp,
    const float* d_parent_conf,
    short* d_disp,
    float* d_disp_float,
    float* d_conf_float,
    size_t left_step_bytes,
    size_t right_step_bytes,
    size_t parent_disp_step_bytes,
    size_t parent_conf_step_bytes,
    size_t disp_step_bytes,
    size_t disp_float_step_bytes,
    size_t conf_float_step_bytes,
    int width, int height,
    int parent_width, int parent_height,
    int numDisparities, int minDisparity, int maxDisparity,
    int blockSize, int P1, int P2,
    int uniquenessRatio, int disp12MaxDiff,
    int preFilterCap,
    int costMode,
    int postFlags,
    int numPaths,
    int refineLevel,
    float minConfidence,
    int adaptiveP2,
    float p2Alpha, float p2Beta, float p2LowerMult, float p2UpperMult,
    cudaStream_t stream);

/*
 * Gaussian [1 4 6 4 1]^2/256 down-sampling by two with BORDER_REFLECT_101
 * (cv::pyrDown for 8-bit single channel).  dst must be
 * ((src_width + 1) / 2, (src_height + 1) / 2); src at least 2x2.
 * Replaces reference include/pyrsgm/pyrsgm_c.h:136-140.
 */
int pyrsgm_pyrdown_u8(
    const unsigned char* d_src, size_t src_step_bytes,
    int src_width, int src_height,
    unsigned char* d_dst, size_t dst_step_bytes,
    int dst_width, int dst_height,
    cudaStream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PYRSGM_C_H */
