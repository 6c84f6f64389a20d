/*
 * pyrsgm_tri3sgm.h -- the two Tri3SGM engine entry points the reference's
 * C API was renamed from (reference README.md:241-252:
 * cuda_3sgm_compute_with_workspace -> pyrsgm_compute_single_scale,
 * cuda_3sgm_compute_pyramid_level_with_workspace -> pyrsgm_compute_level),
 * so a Tri3SGM-style multi-camera pipeline links against this library
 * without renaming its calls.
 *
 * Same arguments, meaning, ownership and return codes as the pyrsgm_c.h
 * functions they forward to; they enqueue exactly the same work.
 *
 * The engine's own device code (LR/LT fusion, LT->LR remap, rotation, depth
 * colouring) was removed from the reference and has no source there, so it
 * is not provided: a pipeline keeps its own.  A vertical (left-top) pair is
 * matched with these calls on images transposed by the caller.
 */
#ifndef PYRSGM_TRI3SGM_H
#define PYRSGM_TRI3SGM_H

#include "pyrsgm_c.h"

#ifdef __cplusplus
extern "C" {
#endif

/* = pyrsgm_compute_single_scale (reference include/pyrsgm/pyrsgm_c.h:63-86). */
int cuda_3sgm_compute_with_workspace(
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

/* = pyrsgm_compute_level (reference include/pyrsgm/pyrsgm_c.h:101-129). */
int cuda_3sgm_compute_pyramid_level_with_workspace(
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

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* PYRSGM_TRI3SGM_H */
