/*
 * sgm_oracle.h -- CPU restatement of the pyrsgm SGM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the parity tests compare the
 * CUDA library against, and the CPU baseline the benchmark reports beside it.
 * The product library never links, loads or calls anything in oracle/.
 *
 * Every function restates one reference kernel or host routine sequentially
 * (same loop order, clamps, sentinels, saturation points, packed-key argmin,
 * right-to-left disparity-2 update order, C truncating division) and cites
 * the reference file:line it follows.  All pointers here are HOST pointers;
 * pitches are in bytes, exactly as in the reference C API.
 *
 * Adaptive P2 (reference src/sgm_kernels.cu:63-74) calls CUDA's __expf, which
 * is not restated on the CPU.  The effective P2 only depends on |dI| in
 * [0,255], so callers pass the 256-entry table produced on the device
 * (p2_lut); with p2_lut == NULL the oracle falls back to libm expf, which is
 * an approximation that is not pinned against the device.
 */
#ifndef PYRSGM_SGM_ORACLE_H
#define PYRSGM_SGM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_workspace orc_workspace;

orc_workspace* orc_create_workspace(void);
void orc_destroy_workspace(orc_workspace* ws);
int orc_workspace_reserve(orc_workspace* ws, int width, int height, int num_disp);

/* Internal volumes of the last call ([y][x][d], int16, d innermost). */
const int16_t* orc_ws_cost(const orc_workspace* ws);   /* d_cost_sad */
const int16_t* orc_ws_acc(const orc_workspace* ws);    /* d_cost_acc */
const int16_t* orc_ws_base(const orc_workspace* ws);   /* d_base_disp */
const uint8_t* orc_ws_valid(const orc_workspace* ws);  /* d_valid_mask */

/* Host adaptive-P2 table for the given parameters using libm expf. */
void orc_p2_table_libm(int P2, float alpha, float beta, float lower, float upper, int* lut256);

int orc_pyrdown_u8(const uint8_t* src, size_t src_step, int src_w, int src_h,
                   uint8_t* dst, size_t dst_step, int dst_w, int dst_h);

int orc_compute_single_scale(
    orc_workspace* ws,
    const uint8_t* left, const uint8_t* right,
    int16_t* disp, float* disp_float, float* conf_float,
    size_t left_step, size_t right_step,
    size_t disp_step, size_t disp_float_step, size_t conf_float_step,
    int width, int height,
    int num_disp, int min_disp,
    int block_size, int P1, int P2,
    int uniqueness, int disp12_max_diff,
    int pre_filter_cap, int cost_mode, int post_flags, int num_paths,
    int adaptive_p2, float p2_alpha, float p2_beta, float p2_lower, float p2_upper,
    const int* p2_lut);

int orc_compute_level(
    orc_workspace* ws,
    const uint8_t* left, const uint8_t* right,
    const int16_t* parent_disp, const float* parent_conf,
    int16_t* disp, float* disp_float, float* conf_float,
    size_t left_step, size_t right_step,
    size_t parent_disp_step, size_t parent_conf_step,
    size_t disp_step, size_t disp_float_step, size_t conf_float_step,
    int width, int height, int parent_width, int parent_height,
    int num_disp, int min_disp, int max_disp,
    int block_size, int P1, int P2,
    int uniqueness, int disp12_max_diff,
    int pre_filter_cap, int cost_mode, int post_flags, int num_paths,
    int refine_level, float min_confidence,
    int adaptive_p2, float p2_alpha, float p2_beta, float p2_lower, float p2_upper,
    const int* p2_lut);

/* pyrsgm::Params restated as a plain struct (reference include/pyrsgm/pyrsgm.h:32-82). */
typedef struct orc_params {
    int num_disparities, min_disparity, block_size, cost_mode;
    int p1, p2, uniqueness_ratio, disp12_max_diff;
    int lr_check, median_filter, num_paths, pre_filter_cap;
    int pyramid_levels, pyramid_coarse_disparities, pyramid_max_disparity;
    float pyramid_min_confidence;
    int adaptive_p2;
    float p2_alpha, p2_beta, p2_lower_mult, p2_upper_mult;
} orc_params;

typedef struct orc_level_info {
    int level, width, height, num_labels, max_disparity, block_size, refine;
} orc_level_info;

void orc_default_params(orc_params* p);
/* Returns 0 and writes the validated params, or -1 (std::invalid_argument). */
int orc_validate_params(const orc_params* in, orc_params* out);
/* Level geometry of StereoMatcher(w, h, p); returns the number of levels or -1. */
int orc_level_geometry(int width, int height, const orc_params* validated, orc_level_info* info5);

/* StereoMatcher::compute restated (reference src/stereo_matcher.cpp:238-338).
 * Outputs may be NULL; pitches in bytes.  Returns 0 or -1. */
int orc_matcher_compute(int width, int height, const orc_params* params,
                        const uint8_t* left, size_t left_step,
                        const uint8_t* right, size_t right_step,
                        int16_t* disp16, size_t disp16_step,
                        float* disp32, size_t disp32_step,
                        float* conf, size_t conf_step,
                        const int* p2_lut);

/* Speckle filter, sequential flood fill: the published semantics of OpenCV's
 * cv::filterSpeckles (calib3d; the reference's bench/pyrsgm_bench.cpp:314
 * passes it to StereoSGBM off).  4-neighbours join one region when neither
 * equals new_val and |a - b| <= max_diff; regions of at most max_size pixels
 * become new_val.  In place; step in bytes.  Returns 0 or -1. */
int orc_filter_speckles(int16_t* img, size_t step, int width, int height, int16_t new_val, int max_size,
                        int max_diff);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int orc_num_threads(void);
void orc_set_num_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
