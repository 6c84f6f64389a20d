/* pyrsgm_io.h -- image and disparity file I/O and Middlebury-style disparity
 * metrics, without OpenCV.  No counterpart in the reference library itself:
 * the reference's benchmark and example carry the same functionality on top
 * of OpenCV (bench/middlebury.h:22-120 readPFM / readNdisp / evaluate,
 * examples/stereo_pair.cpp:37-44 writePfm).
 *
 * All functions are host-only and thread-safe; images are row-major with
 * the given row pitch in elements.  Return 0 on success, -1 on failure with
 * a message in err (if err is non-null).
 */
#ifndef PYRSGM_IO_H
#define PYRSGM_IO_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Grayscale PFM ("Pf"): read into a float buffer the caller allocates after
 * a size query (pass data = NULL to get width/height only).  Both byte
 * orders (scale sign) are accepted; rows are stored bottom-up in the file.
 * Unknown pixels (inf) are kept. */
int pyrsgm_gb300_read_pfm(const char* path, float* data, size_t pitch, int* width, int* height, char* err,
                          size_t err_len);
/* Write little-endian grayscale PFM (scale -1.0), bottom row first. */
int pyrsgm_gb300_write_pfm(const char* path, const float* data, size_t pitch, int width, int height, char* err,
                           size_t err_len);

/* Binary 8-bit PGM ("P5", maxval <= 255), same size-query convention. */
int pyrsgm_gb300_read_pgm(const char* path, unsigned char* data, size_t pitch, int* width, int* height, char* err,
                          size_t err_len);
int pyrsgm_gb300_write_pgm(const char* path, const unsigned char* data, size_t pitch, int width, int height,
                           char* err, size_t err_len);

/* "ndisp=" of a MiddEval3 calib.txt; 0 if absent or unreadable. */
int pyrsgm_gb300_read_ndisp(const char* path);

/* Disparity metrics against ground truth.  disp: float pixels, <= 0 invalid.
 * gt: float, non-finite or <= 0 or > max_disp = unknown (not evaluated).
 * mask: optional 8-bit (255 = evaluate), NULL evaluates every known pixel.
 * Errors |d - gt| count over valid estimates; bad1_all / bad2_all count the
 * invalid estimates as bad too (MiddEval3 convention). */
typedef struct pyrsgm_gb300_metrics {
    int evaluated;   /* ground-truth pixels used */
    int valid;       /* of those, with a valid estimate */
    double avg_err, rms_err;
    double bad05, bad1, bad2, bad4;   /* % of valid pixels with error > 0.5 / 1 / 2 / 4 */
    double density, invalid;          /* valid / evaluated %, and 100 - density */
    double bad1_all, bad2_all;        /* % of evaluated pixels invalid or with error > 1 / 2 */
} pyrsgm_gb300_metrics;

int pyrsgm_gb300_evaluate(const float* disp, size_t disp_pitch, const float* gt, size_t gt_pitch,
                          const unsigned char* mask, size_t mask_pitch, int width, int height, float max_disp,
                          pyrsgm_gb300_metrics* out);

#ifdef __cplusplus
}
#endif

#endif /* PYRSGM_IO_H */
