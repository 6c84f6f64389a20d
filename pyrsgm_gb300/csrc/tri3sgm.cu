// tri3sgm.cu -- the Tri3SGM engine's names for the single-scale and
// per-level entry points (reference README.md:241-252), forwarding to the
// pyrsgm_c.h functions with the same arguments.
#include "pyrsgm/pyrsgm_tri3sgm.h"

extern "C" int cuda_3sgm_compute_with_workspace(
    void* workspace, const unsigned char* d_left_gray, const unsigned char* d_right_gray, short* d_disp,
    float* d_disp_float, float* d_conf_float, size_t left_step_bytes, size_t right_step_bytes,
    size_t disp_step_bytes, size_t disp_float_step_bytes, size_t conf_float_step_bytes, int width, int height,
    int numDisparities, int minDisparity, int blockSize, int P1, int P2, int uniquenessRatio, int disp12MaxDiff,
    int preFilterCap, int costMode, int postFlags, int numPaths, int adaptiveP2, float p2Alpha, float p2Beta,
    float p2LowerMult, float p2UpperMult, cudaStream_t stream)
{
    return pyrsgm_compute_single_scale(workspace, d_left_gray, d_right_gray, d_disp, d_disp_float, d_conf_float,
                                       left_step_bytes, right_step_bytes, disp_step_bytes, disp_float_step_bytes,
                                       conf_float_step_bytes, width, height, numDisparities, minDisparity, blockSize,
                                       P1, P2, uniquenessRatio, disp12MaxDiff, preFilterCap, costMode, postFlags,
                                       numPaths, adaptiveP2, p2Alpha, p2Beta, p2LowerMult, p2UpperMult, stream);
}

extern "C" int cuda_3sgm_compute_pyramid_level_with_workspace(
    void* workspace, const unsigned char* d_left_gray, const unsigned char* d_right_gray, const short* d_parent_disp,
    const float* d_parent_conf, short* d_disp, float* d_disp_float, float* d_conf_float, size_t left_step_bytes,
    size_t right_step_bytes, size_t parent_disp_step_bytes, size_t parent_conf_step_bytes, size_t disp_step_bytes,
    size_t disp_float_step_bytes, size_t conf_float_step_bytes, int width, int height, int parent_width,
    int parent_height, int numDisparities, int minDisparity, int maxDisparity, int blockSize, int P1, int P2,
    int uniquenessRatio, int disp12MaxDiff, int preFilterCap, int costMode, int postFlags, int numPaths,
    int refineLevel, float minConfidence, int adaptiveP2, float p2Alpha, float p2Beta, float p2LowerMult,
    float p2UpperMult, cudaStream_t stream)
{
    return pyrsgm_compute_level(workspace, d_left_gray, d_right_gray, d_parent_disp, d_parent_conf, d_disp,
                                d_disp_float, d_conf_float, left_step_bytes, right_step_bytes, parent_disp_step_bytes,
                                parent_conf_step_bytes, disp_step_bytes, disp_float_step_bytes, conf_float_step_bytes,
                                width, height, parent_width, parent_height, numDisparities, minDisparity,
                                maxDisparity, blockSize, P1, P2, uniquenessRatio, disp12MaxDiff, preFilterCap,
                                costMode, postFlags, numPaths, refineLevel, minConfidence, adaptiveP2, p2Alpha,
                                p2Beta, p2LowerMult, p2UpperMult, stream);
}
