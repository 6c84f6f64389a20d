/*
 * sgm_oracle.c -- CPU restatement of the pyrsgm SGM hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline); the
 * product library never links or calls this file.
 *
 * Citations are reference paths (project-relative) with line numbers.  Each
 * restated kernel runs its CUDA grid sequentially: one loop iteration per
 * block/thread, with the per-block serial loops in the same order, so the
 * integer arithmetic and the tie rules are those of the reference.  Rows
 * (or columns) that the reference runs as independent blocks are spread
 * over OpenMP threads; no result depends on that split.
 *
 * Build with -ffp-contract=off: the few float expressions (confidence,
 * disp/16) must round exactly like the device code, which has no
 * multiply-add in them.
 */
#include "sgm_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define SMAX SHRT_MAX
#define COST_BT 0
#define COST_CENSUS 1
#define POST_LRCHECK 1
#define POST_MEDIAN 2

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int iclamp(int v, int lo, int hi) { return imin(imax(v, lo), hi); }
/* dev_saturate_short, src/sgm_kernels.cu:49-51 */
static inline int16_t sat16(int v) { return (int16_t)imin(SHRT_MAX, imax(SHRT_MIN, v)); }

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Workspace: the 13 buffers of PyrsgmWorkspace, src/sgm_kernels.cu:1486-1503 */
/* ------------------------------------------------------------------------ */
struct orc_workspace {
    int width, height, disp;
    uint8_t *grad1, *grad2;
    uint32_t *census1, *census2;
    int16_t *cost_sad, *cost_acc;
    int16_t *disp_raw, *disp_med, *disp2, *disp2_cost;
    float* conf_raw;
    int16_t* base_disp;
    uint8_t* valid_mask;
};

orc_workspace* orc_create_workspace(void)
{
    return (orc_workspace*)calloc(1, sizeof(orc_workspace));
}

static void ws_release(orc_workspace* ws)
{
    free(ws->grad1); free(ws->grad2); free(ws->census1); free(ws->census2);
    free(ws->cost_sad); free(ws->cost_acc); free(ws->disp_raw); free(ws->disp_med);
    free(ws->disp2); free(ws->disp2_cost); free(ws->conf_raw); free(ws->base_disp);
    free(ws->valid_mask);
    memset(ws, 0, sizeof(*ws));
}

void orc_destroy_workspace(orc_workspace* ws)
{
    if (!ws) return;
    ws_release(ws);
    free(ws);
}

/* pyrsgm_ensure_workspace, src/sgm_kernels.cu:1553-1605 (zero-filled here;
 * the reference leaves fresh device memory undefined). */
static int ws_ensure(orc_workspace* ws, int w, int h, int D)
{
    if (!ws) return -1;
    if (ws->width == w && ws->height == h && ws->disp == D && ws->cost_sad) return 0;
    ws_release(ws);
    size_t px = (size_t)w * h;
    ws->grad1 = calloc(px, 1); ws->grad2 = calloc(px, 1);
    ws->census1 = calloc(px, 4); ws->census2 = calloc(px, 4);
    ws->cost_sad = calloc(px * D, 2); ws->cost_acc = calloc(px * D, 2);
    ws->disp_raw = calloc(px, 2); ws->disp_med = calloc(px, 2);
    ws->disp2 = calloc(px, 2); ws->disp2_cost = calloc(px, 2);
    ws->conf_raw = calloc(px, 4); ws->base_disp = calloc(px, 2);
    ws->valid_mask = calloc(px, 1);
    if (!ws->grad1 || !ws->grad2 || !ws->census1 || !ws->census2 || !ws->cost_sad ||
        !ws->cost_acc || !ws->disp_raw || !ws->disp_med || !ws->disp2 || !ws->disp2_cost ||
        !ws->conf_raw || !ws->base_disp || !ws->valid_mask) {
        ws_release(ws);
        return -1;
    }
    ws->width = w; ws->height = h; ws->disp = D;
    return 0;
}

/* pyrsgm_workspace_reserve, src/sgm_kernels.cu:1607-1615 */
int orc_workspace_reserve(orc_workspace* ws, int w, int h, int D)
{
    if (!ws || w <= 0 || h <= 0 || D <= 0 || D > 1024 || (D % 16) != 0) return -1;
    return ws_ensure(ws, w, h, D);
}

const int16_t* orc_ws_cost(const orc_workspace* ws) { return ws->cost_sad; }
const int16_t* orc_ws_acc(const orc_workspace* ws) { return ws->cost_acc; }
const int16_t* orc_ws_base(const orc_workspace* ws) { return ws->base_disp; }
const uint8_t* orc_ws_valid(const orc_workspace* ws) { return ws->valid_mask; }

/* ------------------------------------------------------------------------ */
/* pyrDown, src/pyrdown.cu:16-74                                             */
/* ------------------------------------------------------------------------ */
static inline int reflect101(int i, int n)
{
    if (i < 0) i = -i;
    if (i >= n) i = 2 * n - 2 - i;
    return i < 0 ? 0 : i;
}

int orc_pyrdown_u8(const uint8_t* src, size_t src_step, int sw, int sh,
                   uint8_t* dst, size_t dst_step, int dw, int dh)
{
    if (!src || !dst || sw < 2 || sh < 2 || dw != (sw + 1) / 2 || dh != (sh + 1) / 2) return -1;
    static const int w5[5] = {1, 4, 6, 4, 1};
#pragma omp parallel for schedule(static)
    for (int y = 0; y < dh; ++y) {
        for (int x = 0; x < dw; ++x) {
            int sum = 0;
            for (int ky = 0; ky < 5; ++ky) {
                const uint8_t* row = src + (size_t)reflect101(2 * y + ky - 2, sh) * src_step;
                int rs = 0;
                for (int kx = 0; kx < 5; ++kx) rs += w5[kx] * (int)row[reflect101(2 * x + kx - 2, sw)];
                sum += w5[ky] * rs;
            }
            dst[(size_t)y * dst_step + x] = (uint8_t)((sum + 128) >> 8);
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Adaptive P2, src/sgm_kernels.cu:63-74, as a table over |dI|                */
/* ------------------------------------------------------------------------ */
void orc_p2_table_libm(int P2, float alpha, float beta, float lower, float upper, int* lut)
{
    for (int diff = 0; diff < 256; ++diff) {
        float ratio = lower + (1.0f + alpha - lower) * expf(-(float)diff / beta);
        float a = (float)P2 * ratio;
        float lo = fmaxf(1.0f, (float)P2 * lower);
        float hi = (float)P2 * upper;
        a = fminf(hi, fmaxf(lo, a));
        lut[diff] = (int)(a + 0.5f);
    }
}

/* The sanitising of src/sgm_kernels.cu:1671-1676 / 1891-1895. */
static void sanitize_p2(int* adaptive, float* alpha, float* beta, float* lower, float* upper)
{
    if (*alpha < 0.0f) *alpha = 0.0f;
    *beta = fmaxf(*beta, 0.5f);
    *upper = fmaxf(*upper, 1.0f);
    *lower = fminf(fmaxf(*lower, 0.0f), *upper);
    if (*alpha <= 0.0f && *lower >= 1.0f) *adaptive = 0;
}

typedef struct { int adaptive; int P2; const int* lut; } p2_ctx;

static inline int p2_eff(const p2_ctx* c, int cur, int prev)
{
    if (!c->adaptive) return c->P2;
    int d = cur - prev;
    return c->lut[d < 0 ? -d : d];
}

/* ------------------------------------------------------------------------ */
/* Per-pixel kernels                                                          */
/* ------------------------------------------------------------------------ */
static void fill16(int16_t* p, size_t n, int16_t v) { for (size_t i = 0; i < n; ++i) p[i] = v; }

/* kernel_BTGradPrecompute, src/sgm_kernels.cu:94-118 */
static void bt_grad(const uint8_t* gray, size_t src_stride, uint8_t* grad, int w, int h, int pfc)
{
    const int ftzero = imax(pfc, 15) | 1;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        const uint8_t* r0 = gray + (size_t)imax(y - 1, 0) * src_stride;
        const uint8_t* r1 = gray + (size_t)y * src_stride;
        const uint8_t* r2 = gray + (size_t)imin(y + 1, h - 1) * src_stride;
        for (int x = 0; x < w; ++x) {
            int xp = imax(x - 1, 0), xn = imin(x + 1, w - 1);
            int g = ((int)r1[xn] - (int)r1[xp]) * 2;
            g += (int)r0[xn] - (int)r0[xp];
            g += (int)r2[xn] - (int)r2[xp];
            if (g < -ftzero) g = -ftzero;
            if (g > ftzero) g = ftzero;
            grad[(size_t)y * w + x] = (uint8_t)(g + ftzero);
        }
    }
}

/* dev_bt_channel_cost, src/sgm_kernels.cu:1002-1028 */
static inline int bt_channel(const uint8_t* lrow, const uint8_t* rrow, int w, int x1, int x2)
{
    if (x2 < 0 || x2 >= w) return 255;
    int u = lrow[x1];
    int ul = (u + lrow[imax(x1 - 1, 0)]) / 2;
    int ur = (u + lrow[imin(x1 + 1, w - 1)]) / 2;
    int u0 = imin(imin(ul, ur), u), u1 = imax(imax(ul, ur), u);
    int v = rrow[x2];
    int vl = (v + rrow[imax(x2 - 1, 0)]) / 2;
    int vr = (v + rrow[imin(x2 + 1, w - 1)]) / 2;
    int v0 = imin(imin(vl, vr), v), v1 = imax(imax(vl, vr), v);
    int c0 = imax(imax(0, u - v1), v0 - u);
    int c1 = imax(imax(0, v - u1), u0 - v);
    return imin(c0, c1);
}

/* dev_bt_pixel_cost, src/sgm_kernels.cu:1030-1043.  kernel_BTCost
 * (src/sgm_kernels.cu:139-239) evaluates the same value through its shared
 * tile (global indices clamped to [0, w-1]), so both stages use this. */
static inline int bt_pixel(const uint8_t* g1, const uint8_t* g2, const uint8_t* i1,
                           const uint8_t* i2, int w, int x, int real_disp)
{
    int x2 = x - real_disp;
    if (x2 < 0 || x2 >= w) return 255;
    int cg = bt_channel(g1, g2, w, x, x2);
    int ci = bt_channel(i1, i2, w, x, x2);
    return imin(255, cg + (ci >> 2));
}

/* kernel_BTCost, src/sgm_kernels.cu:139-239 */
static void bt_cost(const uint8_t* g1, const uint8_t* g2, const uint8_t* i1, size_t s1,
                    const uint8_t* i2, size_t s2, int16_t* cost, int w, int h, int D, int minD)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        const uint8_t* gr1 = g1 + (size_t)y * w; const uint8_t* gr2 = g2 + (size_t)y * w;
        const uint8_t* ir1 = i1 + (size_t)y * s1; const uint8_t* ir2 = i2 + (size_t)y * s2;
        for (int x = 0; x < w; ++x)
            for (int d = 0; d < D; ++d)
                cost[((size_t)y * w + x) * D + d] = (int16_t)bt_pixel(gr1, gr2, ir1, ir2, w, x, d + minD);
    }
}

/* kernel_BoxFilterH, src/sgm_kernels.cu:354-379 (sliding sum == clamped window sum) */
static void box_h(const int16_t* src, int16_t* dst, int w, int h, int D, int bs)
{
    const int half = bs / 2;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        const int16_t* s = src + (size_t)y * w * D;
        int16_t* o = dst + (size_t)y * w * D;
        for (int d = 0; d < D; ++d) {
            int sum = 0;
            for (int k = -half; k <= half; ++k) sum += s[(size_t)iclamp(k, 0, w - 1) * D + d];
            o[d] = (int16_t)imin(SMAX, sum);
            for (int x = 1; x < w; ++x) {
                int lx = iclamp(x - 1 - half, 0, w - 1), ex = iclamp(x + half, 0, w - 1);
                sum += (int)s[(size_t)ex * D + d] - (int)s[(size_t)lx * D + d];
                o[(size_t)x * D + d] = (int16_t)imin(SMAX, sum);
            }
        }
    }
}

/* kernel_BoxFilterV, src/sgm_kernels.cu:390-416 */
static void box_v(const int16_t* src, int16_t* dst, int w, int h, int D, int bs)
{
    const int half = bs / 2;
    const size_t stride = (size_t)w * D;
#pragma omp parallel for schedule(static)
    for (int x = 0; x < w; ++x) {
        for (int d = 0; d < D; ++d) {
            size_t col = (size_t)x * D + d;
            int sum = 0;
            for (int k = -half; k <= half; ++k) sum += src[(size_t)iclamp(k, 0, h - 1) * stride + col];
            dst[col] = (int16_t)imin(SMAX, sum);
            for (int y = 1; y < h; ++y) {
                int ly = iclamp(y - 1 - half, 0, h - 1), ey = iclamp(y + half, 0, h - 1);
                sum += (int)src[(size_t)ey * stride + col] - (int)src[(size_t)ly * stride + col];
                dst[(size_t)y * stride + col] = (int16_t)imin(SMAX, sum);
            }
        }
    }
}

/* kernel_CensusCompute, src/sgm_kernels.cu:251-298 (5x5, replicate borders,
 * MSB first, dy-major, bit = neighbour < centre) */
static void census(const uint8_t* gray, size_t stride, uint32_t* out, int w, int h)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            const uint8_t c = gray[(size_t)y * stride + x];
            uint32_t cv = 0;
            for (int dy = 0; dy < 5; ++dy) {
                const uint8_t* row = gray + (size_t)iclamp(y + dy - 2, 0, h - 1) * stride;
                for (int dx = 0; dx < 5; ++dx) {
                    cv <<= 1;
                    cv |= (uint32_t)(row[iclamp(x + dx - 2, 0, w - 1)] < c);
                }
            }
            out[(size_t)y * w + x] = cv;
        }
    }
}

static inline int popc32(uint32_t v) { return __builtin_popcount(v); }

/* kernel_CensusCost, src/sgm_kernels.cu:303-327 */
static void census_cost(const uint32_t* cl, const uint32_t* cr, int16_t* cost, int w, int h, int D, int minD)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            for (int d = 0; d < D; ++d) {
                int x2 = x - (d + minD);
                int c = 24;
                if (x2 >= 0 && x2 < w) c = popc32(cl[(size_t)y * w + x] ^ cr[(size_t)y * w + x2]);
                cost[((size_t)y * w + x) * D + d] = (int16_t)c;
            }
}

/* ------------------------------------------------------------------------ */
/* Single-scale path kernels                                                  */
/* ------------------------------------------------------------------------ */

/* One recurrence step shared by the three single-scale path kernels
 * (src/sgm_kernels.cu:560-565, 623-628, 727-732). */
static inline void ss_step(const int16_t* Lp, int16_t* Lc, const int16_t* C, int D,
                           int P1, int p2, int minPrev)
{
    for (int d = 0; d < D; ++d) {
        int Lm = d > 0 ? (int)Lp[d - 1] + P1 : SMAX;
        int Ls = Lp[d];
        int Lpl = d < D - 1 ? (int)Lp[d + 1] + P1 : SMAX;
        int Lj = imin(SMAX, minPrev + p2);
        int best = imin(imin(Lm, Lpl), imin(Ls, Lj));
        Lc[d] = sat16((int)C[d] + best - minPrev);
    }
}

static inline int vmin16(const int16_t* v, int D)
{
    int m = v[0];
    for (int d = 1; d < D; ++d) m = imin(m, v[d]);
    return (int16_t)m;
}

/* kernel_SGM_PathLR, src/sgm_kernels.cu:520-578 */
static void ss_path_lr(int16_t* acc, const int16_t* C, const uint8_t* img, size_t img_stride,
                       int w, int h, int D, int startX, int endX, int P1, const p2_ctx* p2)
{
    if (startX < 0) startX = 0;
    if (endX > w) endX = w;
    if (startX >= endX) return;
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
#pragma omp for schedule(static)
        for (int y = 0; y < h; ++y) {
            int16_t *Lp = buf, *Lc = buf + D;
            size_t rb = (size_t)y * w * D;
            const uint8_t* ir = img + (size_t)y * img_stride;
            for (int d = 0; d < D; ++d) Lp[d] = C[rb + (size_t)startX * D + d];
            int minP = vmin16(Lp, D);
            for (int d = 0; d < D; ++d) acc[rb + (size_t)startX * D + d] = Lp[d];
            for (int x = startX + 1; x < endX; ++x) {
                ss_step(Lp, Lc, C + rb + (size_t)x * D, D, P1, p2_eff(p2, ir[x], ir[x - 1]), minP);
                minP = vmin16(Lc, D);
                for (int d = 0; d < D; ++d) acc[rb + (size_t)x * D + d] = Lc[d];
                int16_t* t = Lp; Lp = Lc; Lc = t;
            }
        }
        free(buf);
    }
}

/* kernel_SGM_PathTB, src/sgm_kernels.cu:587-638 */
static void ss_path_tb(int16_t* acc, const int16_t* C, const uint8_t* img, size_t img_stride,
                       int w, int h, int D, int P1, const p2_ctx* p2)
{
    const size_t stride = (size_t)w * D;
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
#pragma omp for schedule(static)
        for (int x = 0; x < w; ++x) {
            int16_t *Lp = buf, *Lc = buf + D;
            for (int d = 0; d < D; ++d) Lp[d] = C[(size_t)x * D + d];
            int minP = vmin16(Lp, D);
            for (int d = 0; d < D; ++d) {
                size_t o = (size_t)x * D + d;
                acc[o] = (int16_t)imin(SMAX, (int)acc[o] + Lp[d]);
            }
            for (int y = 1; y < h; ++y) {
                int p2v = p2_eff(p2, img[(size_t)y * img_stride + x], img[(size_t)(y - 1) * img_stride + x]);
                ss_step(Lp, Lc, C + (size_t)y * stride + (size_t)x * D, D, P1, p2v, minP);
                minP = vmin16(Lc, D);
                for (int d = 0; d < D; ++d) {
                    size_t o = (size_t)y * stride + (size_t)x * D + d;
                    acc[o] = (int16_t)imin(SMAX, (int)acc[o] + Lc[d]);
                }
                int16_t* t = Lp; Lp = Lc; Lc = t;
            }
        }
        free(buf);
    }
}

/* kernel_SGM_PathRL_WTA, src/sgm_kernels.cu:665-819 */
static void ss_path_rl_wta(int16_t* acc, const int16_t* C, const uint8_t* img, size_t img_stride,
                           int16_t* disp, int16_t* disp2, int16_t* disp2_cost, float* conf,
                           int w, int h, int D, int minD, int P1, int uniq, int accumulate,
                           const p2_ctx* p2)
{
    const int16_t invalid = (int16_t)((minD - 1) * 16);
    const int minX1 = imax(minD + D, 0);
    const int maxX1 = w + imin(minD, 0);
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
#pragma omp for schedule(static)
        for (int y = 0; y < h; ++y) {
            int16_t *Lp = buf, *Lc = buf + D;
            size_t rb = (size_t)y * w * D;
            const uint8_t* ir = img + (size_t)y * img_stride;
            int xs = w - 1;
            for (int d = 0; d < D; ++d) Lp[d] = C[rb + (size_t)xs * D + d];
            int minP = vmin16(Lp, D);
            for (int d = 0; d < D; ++d) {
                size_t o = rb + (size_t)xs * D + d;
                acc[o] = (int16_t)imin(SMAX, (accumulate ? (int)acc[o] : 0) + Lp[d]);
            }
            disp[(size_t)y * w + xs] = invalid;
            conf[(size_t)y * w + xs] = 0.0f;
            for (int x = w - 2; x >= 0; --x) {
                const size_t xb = rb + (size_t)x * D;
                ss_step(Lp, Lc, C + xb, D, P1, p2_eff(p2, ir[x], ir[x + 1]), minP);
                minP = vmin16(Lc, D);
                /* accumulate + packed (cost<<16 | d) argmin, src/sgm_kernels.cu:739-753 */
                unsigned best_key = 0xFFFFFFFFu;
                for (int d = 0; d < D; ++d) {
                    int total = (accumulate ? (int)acc[xb + d] : 0) + Lc[d];
                    int16_t my = (int16_t)imin(SMAX, total);
                    acc[xb + d] = my;
                    unsigned key = ((unsigned)(uint16_t)my << 16) | (unsigned)d;
                    if (key < best_key) best_key = key;
                }
                int16_t min_cost = (int16_t)(best_key >> 16);
                int16_t best_d = (int16_t)(best_key & 0xFFFFu);
                int alt = SMAX;
                for (int d = 0; d < D; ++d)
                    if (abs(d - (int)best_d) > 1) alt = imin(alt, acc[xb + d]);
                int16_t alt_cost = (int16_t)alt;
                size_t px = (size_t)y * w + x;
                if (x < minX1 || x >= maxX1) {
                    disp[px] = invalid;
                    conf[px] = 0.0f;
                } else {
                    int unique = 1;
                    if (uniq > 0 && min_cost < SMAX / 2) {
                        if ((int)alt_cost * (100 - uniq) < (int)min_cost * 100) unique = 0;
                    }
                    if (unique && min_cost < SMAX / 2) {
                        int d_int;
                        if (best_d > 0 && best_d < D - 1) {
                            int16_t c0 = acc[xb + best_d - 1], c1 = acc[xb + best_d], c2 = acc[xb + best_d + 1];
                            int den = imax((int)c0 + c2 - 2 * (int)c1, 1);
                            d_int = best_d * 16 + ((int)(c0 - c2) * 16 + den) / (den * 2);
                        } else {
                            d_int = best_d * 16;
                        }
                        int16_t d_val = (int16_t)(d_int + minD * 16);
                        int x2 = x - best_d - minD;
                        if (x2 >= 0 && x2 < w) {
                            size_t o = (size_t)y * w + x2;
                            if (disp2_cost[o] > min_cost) {
                                disp2_cost[o] = min_cost;
                                disp2[o] = (int16_t)(best_d + minD);
                            }
                        }
                        disp[px] = d_val;
                        float den_f = fmaxf((float)min_cost, 1.0f);
                        float c = ((float)alt_cost - (float)min_cost) / den_f;
                        conf[px] = fminf(fmaxf(c, 0.0f), 1.0f);
                    } else {
                        disp[px] = invalid;
                        conf[px] = 0.0f;
                    }
                }
                int16_t* t = Lp; Lp = Lc; Lc = t;
            }
        }
        free(buf);
    }
}

/* kernel_PseudoLRCheck, src/sgm_kernels.cu:825-851 */
static void pseudo_lr_check(int16_t* disp, const int16_t* disp2, float* conf, int w, int h, int minD, int maxdiff)
{
    const int16_t invalid = (int16_t)((minD - 1) * 16);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t i = (size_t)y * w + x;
            int d1 = disp[i];
            if (d1 == invalid) continue;
            int d0 = d1 >> 4, dc = (d1 + 15) >> 4;
            int xa = x - d0, xb = x - dc;
            const int16_t* r = disp2 + (size_t)y * w;
            if (0 <= xa && xa < w && r[xa] >= minD && abs(r[xa] - d0) > maxdiff &&
                0 <= xb && xb < w && r[xb] >= minD && abs(r[xb] - dc) > maxdiff) {
                disp[i] = invalid;
                conf[i] = 0.0f;
            }
        }
}

/* kernel_StrictPyramidLRCheck, src/sgm_kernels.cu:855-889 */
static void strict_lr_check(int16_t* disp, const int16_t* disp2, float* conf, int w, int h, int minD, int maxdiff)
{
    const int16_t invalid = (int16_t)((minD - 1) * 16);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t p = (size_t)y * w + x;
            int d16 = disp[p];
            if (d16 == invalid) continue;
            int d0 = d16 >> 4, d1 = (d16 + 15) >> 4;
            int r0 = x - d0, r1 = x - d1;
            const int16_t* r = disp2 + (size_t)y * w;
            int ok = 0;
            if (r0 >= 0 && r0 < w && r[r0] >= minD && abs((int)r[r0] - d0) <= maxdiff) ok = 1;
            if (r1 >= 0 && r1 < w && r[r1] >= minD && abs((int)r[r1] - d1) <= maxdiff) ok = 1;
            if (!ok) { disp[p] = invalid; conf[p] = 0.0f; }
        }
}

/* kernel_MedianFilter3x3 + kernel_ClearChangedMedianConfidence,
 * src/sgm_kernels.cu:891-931 */
static void median3x3(const int16_t* src, int16_t* dst, float* conf, int w, int h)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int16_t v[9];
            int n = 0;
            for (int dy = -1; dy <= 1; ++dy) {
                int yy = y + dy;
                if (yy < 0 || yy >= h) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    int xx = x + dx;
                    if (xx < 0 || xx >= w) continue;
                    v[n++] = src[(size_t)yy * w + xx];
                }
            }
            for (int i = 1; i < n; ++i) {
                int16_t k = v[i];
                int j = i - 1;
                while (j >= 0 && v[j] > k) { v[j + 1] = v[j]; --j; }
                v[j + 1] = k;
            }
            dst[(size_t)y * w + x] = v[n / 2];
        }
    for (size_t p = 0; p < (size_t)w * h; ++p)
        if (src[p] != dst[p]) conf[p] = 0.0f;
}

/* ------------------------------------------------------------------------ */
/* Pyramid helpers and kernels                                                */
/* ------------------------------------------------------------------------ */

/* kernel_PrepareRefineLabels, src/sgm_kernels.cu:955-1000 */
static void prepare_refine_labels(const int16_t* pdisp, const float* pconf, int pw, int ph,
                                  int pd_pitch, int pc_pitch, int16_t* base, uint8_t* valid,
                                  int w, int h, int minD, int maxD, int localD, float minConf)
{
    const int16_t pinv = (int16_t)((minD - 1) * 16);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int px = imin(x >> 1, pw - 1), py = imin(y >> 1, ph - 1);
            int16_t raw = pdisp[(size_t)py * pd_pitch + px];
            float c = pconf[(size_t)py * pc_pitch + px];
            size_t o = (size_t)y * w + x;
            if (raw == pinv || c < minConf) { base[o] = (int16_t)minD; valid[o] = 0; continue; }
            int pred16 = (int)raw * 2;
            int center = (pred16 + 8) >> 4;
            int resid = pred16 - center * 16;
            int b = center + (resid < 0 ? -(localD / 2) : -(localD / 2) + 1);
            int physMax = imin(maxD, x);
            int largest = physMax - localD + 1;
            if (largest >= minD) b = imin(imax(b, minD), largest);
            else b = minD;
            base[o] = (int16_t)b;
            valid[o] = 1;
        }
}

/* dev_bt_pixel_cost window sum, kernel_BTWindowCostLocal, src/sgm_kernels.cu:1075-1110;
 * label validity dev_pyramid_label_geometry_valid, src/sgm_kernels.cu:1045-1054 */
static inline int geom_valid(const uint8_t* valid, const int16_t* base, size_t p, int x, int d,
                             int D, int minD, int maxD, int w)
{
    if (!valid[p] || d < 0 || d >= D) return 0;
    int r = (int)base[p] + d;
    int x2 = x - r;
    return r >= minD && r <= maxD && x2 >= 0 && x2 < w;
}

static void bt_window_cost_local(const uint8_t* g1, const uint8_t* g2, const uint8_t* i1, size_t s1,
                                 const uint8_t* i2, size_t s2, const int16_t* base, const uint8_t* valid,
                                 int16_t* cost, int w, int h, int D, int minD, int maxD, int bs)
{
    const int half = bs / 2;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t p = (size_t)y * w + x;
            for (int d = 0; d < D; ++d) {
                size_t o = p * D + d;
                if (!geom_valid(valid, base, p, x, d, D, minD, maxD, w)) { cost[o] = SMAX; continue; }
                int r = (int)base[p] + d;
                int sum = 0;
                for (int dy = -half; dy <= half; ++dy) {
                    int yy = iclamp(y + dy, 0, h - 1);
                    const uint8_t* gr1 = g1 + (size_t)yy * w; const uint8_t* gr2 = g2 + (size_t)yy * w;
                    const uint8_t* ir1 = i1 + (size_t)yy * s1; const uint8_t* ir2 = i2 + (size_t)yy * s2;
                    for (int dx = -half; dx <= half; ++dx) {
                        int xx = iclamp(x + dx, 0, w - 1);
                        sum += bt_pixel(gr1, gr2, ir1, ir2, w, xx, r);
                    }
                }
                cost[o] = (int16_t)imin(sum, SMAX - 1);
            }
        }
}

/* kernel_CensusCostLocal, src/sgm_kernels.cu:1112-1133 */
static void census_cost_local(const uint32_t* cl, const uint32_t* cr, const int16_t* base,
                              const uint8_t* valid, int16_t* cost, int w, int h, int D, int minD, int maxD)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            size_t p = (size_t)y * w + x;
            for (int d = 0; d < D; ++d) {
                int x2 = x - ((int)base[p] + d);
                cost[p * D + d] = geom_valid(valid, base, p, x, d, D, minD, maxD, w)
                    ? (int16_t)popc32(cl[(size_t)y * w + x] ^ cr[(size_t)y * w + x2]) : (int16_t)SMAX;
            }
        }
}

/* dev_pyramid_valid_label_count, src/sgm_kernels.cu:1059-1070 */
static inline int valid_count(const uint8_t* valid, const int16_t* base, size_t p, int x,
                              int D, int minD, int maxD, int w)
{
    if (!valid[p] || D <= 0) return 0;
    int b = base[p];
    int first = imax(minD, x - (w - 1)), last = imin(maxD, x);
    int fl = imax(0, first - b), ll = imin(D - 1, last - b);
    return ll >= fl ? ll - fl + 1 : 0;
}

/* The pyramid recurrence of one pixel, shared by src/sgm_kernels.cu:1230-1252,
 * 1299-1322 and 1382-1404.  lv[d] = dev_pyramid_label_valid. */
static inline void pyr_step(const int16_t* Lp, int16_t* Lc, const int16_t* C, const uint8_t* lv,
                            int D, int base, int prevBase, int prevActive, int P1, int p2, int minPrev)
{
    for (int d = 0; d < D; ++d) {
        int c = lv[d] ? (int)C[d] : SMAX;
        if (!prevActive) { Lc[d] = (int16_t)c; continue; }
        if (!lv[d]) { Lc[d] = SMAX; continue; }
        int same = d + base - prevBase;
        int l0 = (same >= 0 && same < D) ? (int)Lp[same] : SMAX;
        int mi = same - 1, pl = same + 1;
        int lm = (mi >= 0 && mi < D && Lp[mi] < SMAX) ? (int)Lp[mi] + P1 : SMAX;
        int lp = (pl >= 0 && pl < D && Lp[pl] < SMAX) ? (int)Lp[pl] + P1 : SMAX;
        int lj = imin(SMAX, minPrev + p2);
        int best = imin(imin(l0, lm), imin(lp, lj));
        Lc[d] = best < SMAX ? sat16(c + best - minPrev) : (int16_t)SMAX;
    }
}

typedef struct {
    int w, h, D, minD, maxD, P1;
    const int16_t* C;
    const int16_t* base;
    const uint8_t* valid;
    const uint8_t* img;
    size_t img_stride;
    const p2_ctx* p2;
} pyr_args;

static inline void label_valid_row(const pyr_args* a, size_t p, int x, uint8_t* lv)
{
    for (int d = 0; d < a->D; ++d)
        lv[d] = (uint8_t)(geom_valid(a->valid, a->base, p, x, d, a->D, a->minD, a->maxD, a->w) &&
                          a->C[p * a->D + d] < SMAX);
}

/* kernel_SGM_PathLRPyramid, src/sgm_kernels.cu:1191-1261 */
static void pyr_path_lr(int16_t* acc, const pyr_args* a)
{
    const int w = a->w, D = a->D;
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
        uint8_t* lv = malloc(D);
#pragma omp for schedule(static)
        for (int y = 0; y < a->h; ++y) {
            int16_t *Lp = buf, *Lc = buf + D;
            int prevActive = 0, prevBase = a->minD, minPrev = SMAX;
            const uint8_t* ir = a->img + (size_t)y * a->img_stride;
            for (int x = 0; x < w; ++x) {
                size_t p = (size_t)y * w + x;
                int base = a->base[p];
                label_valid_row(a, p, x, lv);
                int vc = valid_count(a->valid, a->base, p, x, D, a->minD, a->maxD, w);
                if (vc == 0) {
                    for (int d = 0; d < D; ++d) { Lc[d] = SMAX; acc[p * D + d] = SMAX; }
                    prevActive = 0;
                    continue;
                }
                int p2v = (prevActive) ? p2_eff(a->p2, ir[x], x > 0 ? ir[x - 1] : 0) : 0;
                pyr_step(Lp, Lc, a->C + p * D, lv, D, base, prevBase, prevActive, a->P1, p2v, minPrev);
                int minCur = vmin16(Lc, D);
                for (int d = 0; d < D; ++d) acc[p * D + d] = Lc[d];
                int16_t* t = Lp; Lp = Lc; Lc = t;
                minPrev = minCur; prevBase = base; prevActive = minCur < SMAX;
            }
        }
        free(buf); free(lv);
    }
}

/* kernel_SGM_PathTBPyramid, src/sgm_kernels.cu:1263-1334 */
static void pyr_path_tb(int16_t* acc, const pyr_args* a)
{
    const int w = a->w, D = a->D;
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
        uint8_t* lv = malloc(D);
#pragma omp for schedule(static)
        for (int x = 0; x < w; ++x) {
            int16_t *Lp = buf, *Lc = buf + D;
            int prevActive = 0, prevBase = a->minD, minPrev = SMAX;
            for (int y = 0; y < a->h; ++y) {
                size_t p = (size_t)y * w + x;
                int base = a->base[p];
                label_valid_row(a, p, x, lv);
                int vc = valid_count(a->valid, a->base, p, x, D, a->minD, a->maxD, w);
                if (vc == 0) {
                    for (int d = 0; d < D; ++d) { Lc[d] = SMAX; acc[p * D + d] = SMAX; }
                    prevActive = 0;
                    continue;
                }
                int p2v = prevActive ? p2_eff(a->p2, a->img[(size_t)y * a->img_stride + x],
                                              y > 0 ? a->img[(size_t)(y - 1) * a->img_stride + x] : 0) : 0;
                pyr_step(Lp, Lc, a->C + p * D, lv, D, base, prevBase, prevActive, a->P1, p2v, minPrev);
                int minCur = vmin16(Lc, D);
                for (int d = 0; d < D; ++d) {
                    int old = acc[p * D + d];
                    acc[p * D + d] = (old < SMAX && Lc[d] < SMAX) ? (int16_t)imin(SMAX - 1, old + (int)Lc[d])
                                                                 : (int16_t)SMAX;
                }
                int16_t* t = Lp; Lp = Lc; Lc = t;
                minPrev = minCur; prevBase = base; prevActive = minCur < SMAX;
            }
        }
        free(buf); free(lv);
    }
}

/* kernel_SGM_PathRLPyramidWTA, src/sgm_kernels.cu:1336-1478 */
static void pyr_path_rl_wta(int16_t* acc, const pyr_args* a, int16_t* disp, int16_t* disp2,
                            int16_t* disp2_cost, float* conf, int uniq, float minConf, int accumulate)
{
    const int w = a->w, D = a->D, minD = a->minD, maxD = a->maxD;
    const int16_t invalid = (int16_t)((minD - 1) * 16);
#pragma omp parallel
    {
        int16_t* buf = malloc(sizeof(int16_t) * 2 * D);
        uint8_t* lv = malloc(D);
#pragma omp for schedule(static)
        for (int y = 0; y < a->h; ++y) {
            int16_t *Lp = buf, *Lc = buf + D;
            int prevActive = 0, prevBase = minD, minPrev = SMAX;
            const uint8_t* ir = a->img + (size_t)y * a->img_stride;
            for (int x = w - 1; x >= 0; --x) {
                size_t p = (size_t)y * w + x;
                int base = a->base[p];
                label_valid_row(a, p, x, lv);
                int vc = valid_count(a->valid, a->base, p, x, D, minD, maxD, w);
                if (vc == 0) {
                    for (int d = 0; d < D; ++d) { Lc[d] = SMAX; acc[p * D + d] = SMAX; }
                    disp[p] = invalid;
                    conf[p] = 0.0f;
                    prevActive = 0;
                    continue;
                }
                int p2v = prevActive ? p2_eff(a->p2, ir[x], x + 1 < w ? ir[x + 1] : 0) : 0;
                pyr_step(Lp, Lc, a->C + p * D, lv, D, base, prevBase, prevActive, a->P1, p2v, minPrev);
                int minCur = vmin16(Lc, D);
                unsigned best_key = 0xFFFFFFFFu;
                for (int d = 0; d < D; ++d) {
                    int old = accumulate ? (int)acc[p * D + d] : 0;
                    int16_t my = (lv[d] && Lc[d] < SMAX && (!accumulate || old < SMAX))
                        ? (int16_t)imin(SMAX - 1, old + (int)Lc[d]) : (int16_t)SMAX;
                    acc[p * D + d] = my;
                    unsigned key = ((unsigned)(uint16_t)my << 16) | (unsigned)d;
                    if (key < best_key) best_key = key;
                }
                int16_t minCost = (int16_t)(best_key >> 16);
                int bestD = (int)(best_key & 0xFFFFu);
                int alt = SMAX;
                for (int d = 0; d < D; ++d)
                    if (lv[d] && abs(d - bestD) > 1) alt = imin(alt, acc[p * D + d]);
                int16_t altCost = (int16_t)alt;

                int ok = vc >= 3 && minCost < SMAX && altCost < SMAX;
                if (ok && uniq > 0 && (int)altCost * (100 - uniq) < (int)minCost * 100) ok = 0;
                const int realBest = base + bestD;
                const int physMax = imin(maxD, x);
                if ((bestD == 0 && base > minD) || (bestD == D - 1 && base + D - 1 < physMax)) ok = 0;
                float c = 0.0f;
                if (ok) {
                    float den = fmaxf((float)minCost, 1.0f);
                    c = fminf(fmaxf(((float)altCost - (float)minCost) / den, 0.0f), 1.0f);
                    if (c < minConf) ok = 0;
                }
                if (ok) {
                    int d16 = realBest * 16;
                    if (bestD > 0 && bestD + 1 < D) {
                        size_t bo = p * D + bestD;
                        int16_t c0 = acc[bo - 1], c1 = acc[bo], c2 = acc[bo + 1];
                        if (c0 < SMAX && c1 < SMAX && c2 < SMAX) {
                            int den2 = imax((int)c0 + c2 - 2 * (int)c1, 1);
                            d16 += ((int)(c0 - c2) * 16 + den2) / (den2 * 2);
                        }
                    }
                    disp[p] = (int16_t)d16;
                    conf[p] = c;
                    int x2 = x - realBest;
                    if (x2 >= 0 && x2 < w) {
                        size_t rp = (size_t)y * w + x2;
                        if (disp2_cost[rp] > minCost) { disp2_cost[rp] = minCost; disp2[rp] = (int16_t)realBest; }
                    }
                } else {
                    disp[p] = invalid;
                    conf[p] = 0.0f;
                }
                int16_t* t = Lp; Lp = Lc; Lc = t;
                minPrev = minCur; prevBase = base; prevActive = minCur < SMAX;
            }
        }
        free(buf); free(lv);
    }
}

/* convertDispAndConfKernel, src/sgm_kernels.cu:1530-1551 */
static void convert_out(const int16_t* d16, const float* craw, float* d32, size_t d32_step,
                        float* c32, size_t c32_step, int w, int h, int16_t invalid)
{
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            int16_t raw = d16[(size_t)y * w + x];
            float d = raw / 16.0f;
            int ok = raw != invalid && d > 0.0f;
            float* pd = (float*)((char*)d32 + (size_t)y * d32_step) + x;
            float* pc = (float*)((char*)c32 + (size_t)y * c32_step) + x;
            *pd = ok ? d : 0.0f;
            *pc = ok ? craw[(size_t)y * w + x] : 0.0f;
        }
}

static void copy2d(void* dst, size_t dstep, const void* src, size_t sstep, size_t row_bytes, int h)
{
    for (int y = 0; y < h; ++y)
        memcpy((char*)dst + (size_t)y * dstep, (const char*)src + (size_t)y * sstep, row_bytes);
}

/* ------------------------------------------------------------------------ */
/* pyrsgm_compute_level, src/sgm_kernels.cu:1617-1862                         */
/* ------------------------------------------------------------------------ */
int orc_compute_level(
    orc_workspace* ws, const uint8_t* left, const uint8_t* right,
    const int16_t* parent_disp, const float* parent_conf,
    int16_t* disp, float* disp_float, float* conf_float,
    size_t left_step, size_t right_step, size_t pd_step, size_t pc_step,
    size_t disp_step, size_t df_step, size_t cf_step,
    int w, int h, int pw, int ph, int D, int minD, int maxD,
    int bs, int P1, int P2, int uniq, int maxdiff, int pfc, int cost_mode,
    int post, int paths, int refine, float minConf,
    int adaptive, float alpha, float beta, float lower, float upper, const int* lut)
{
    if (!ws || !left || !right || w <= 0 || h <= 0 || D <= 0 || D > 1024 || (D % 16) != 0 ||
        (refine && D > 256))
        return -1;
    if (refine && (!parent_disp || !parent_conf || pw <= 0 || ph <= 0)) return -1;
    maxD = imin(maxD, w - 1);
    maxD = imin(maxD, SMAX / 16);
    if (!refine) maxD = imin(maxD, minD + D - 1);
    if (maxD < minD || ws_ensure(ws, w, h, D) != 0) return -1;

    sanitize_p2(&adaptive, &alpha, &beta, &lower, &upper);
    minConf = fminf(fmaxf(minConf, 0.0f), 1.0f);
    if (paths < 1) paths = 1;
    if (paths > 3) paths = 3;
    int tbl[256];
    if (adaptive && !lut) { orc_p2_table_libm(P2, alpha, beta, lower, upper, tbl); lut = tbl; }
    p2_ctx p2 = {adaptive, P2, lut};

    const size_t px = (size_t)w * h;
    const int16_t invalid = (int16_t)((minD - 1) * 16);
    fill16(ws->disp_raw, px, invalid);
    fill16(ws->disp2, px, invalid);
    fill16(ws->disp2_cost, px, SMAX);
    memset(ws->conf_raw, 0, px * sizeof(float));

    if (refine) {
        prepare_refine_labels(parent_disp, parent_conf, pw, ph, (int)(pd_step / 2), (int)(pc_step / 4),
                              ws->base_disp, ws->valid_mask, w, h, minD, maxD, D, minConf);
    } else {
        fill16(ws->base_disp, px, (int16_t)minD);       /* kernel_InitCoarseLabels */
        memset(ws->valid_mask, 1, px);
    }

    if (cost_mode == COST_CENSUS) {
        census(left, left_step, ws->census1, w, h);
        census(right, right_step, ws->census2, w, h);
        if (refine)
            census_cost_local(ws->census1, ws->census2, ws->base_disp, ws->valid_mask, ws->cost_sad,
                              w, h, D, minD, maxD);
        else
            census_cost(ws->census1, ws->census2, ws->cost_sad, w, h, D, minD);
    } else {
        bt_grad(left, left_step, ws->grad1, w, h, pfc);
        bt_grad(right, right_step, ws->grad2, w, h, pfc);
        if (refine) {
            bt_window_cost_local(ws->grad1, ws->grad2, left, left_step, right, right_step,
                                 ws->base_disp, ws->valid_mask, ws->cost_sad, w, h, D, minD, maxD, bs);
        } else {
            bt_cost(ws->grad1, ws->grad2, left, left_step, right, right_step, ws->cost_sad, w, h, D, minD);
            box_h(ws->cost_sad, ws->cost_acc, w, h, D, bs);
            box_v(ws->cost_acc, ws->cost_sad, w, h, D, bs);
        }
    }

    pyr_args a = {w, h, D, minD, maxD, P1, ws->cost_sad, ws->base_disp, ws->valid_mask, left, left_step, &p2};
    if (paths >= 2) pyr_path_lr(ws->cost_acc, &a);
    if (paths >= 3) pyr_path_tb(ws->cost_acc, &a);
    pyr_path_rl_wta(ws->cost_acc, &a, ws->disp_raw, ws->disp2, ws->disp2_cost, ws->conf_raw,
                    uniq, minConf, paths >= 2 ? 1 : 0);

    if (post & POST_LRCHECK) strict_lr_check(ws->disp_raw, ws->disp2, ws->conf_raw, w, h, minD, maxdiff);
    int16_t* fin = ws->disp_raw;
    if (post & POST_MEDIAN) {
        median3x3(ws->disp_raw, ws->disp_med, ws->conf_raw, w, h);
        fin = ws->disp_med;
    }
    if (disp) copy2d(disp, disp_step, fin, (size_t)w * 2, (size_t)w * 2, h);
    if (disp_float && conf_float)
        convert_out(fin, ws->conf_raw, disp_float, df_step, conf_float, cf_step, w, h, invalid);
    else if (conf_float)
        copy2d(conf_float, cf_step, ws->conf_raw, (size_t)w * 4, (size_t)w * 4, h);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* pyrsgm_compute_single_scale, src/sgm_kernels.cu:1864-2076                  */
/* ------------------------------------------------------------------------ */
int orc_compute_single_scale(
    orc_workspace* ws, const uint8_t* left, const uint8_t* right,
    int16_t* disp, float* disp_float, float* conf_float,
    size_t left_step, size_t right_step, size_t disp_step, size_t df_step, size_t cf_step,
    int w, int h, int D, int minD, int bs, int P1, int P2, int uniq, int maxdiff,
    int pfc, int cost_mode, int post, int paths,
    int adaptive, float alpha, float beta, float lower, float upper, const int* lut)
{
    sanitize_p2(&adaptive, &alpha, &beta, &lower, &upper);
    const int minX1 = imax(minD + D, 0);
    const int maxX1 = w + imin(minD, 0);
    if (paths < 1) paths = 1;
    if (paths > 3) paths = 3;
    if (ws_ensure(ws, w, h, D) != 0) return -1;
    int tbl[256];
    if (adaptive && !lut) { orc_p2_table_libm(P2, alpha, beta, lower, upper, tbl); lut = tbl; }
    p2_ctx p2 = {adaptive, P2, lut};

    const size_t px = (size_t)w * h;
    const int16_t invalid = (int16_t)((minD - 1) * 16);
    fill16(ws->disp_raw, px, invalid);
    fill16(ws->disp2, px, invalid);
    fill16(ws->disp2_cost, px, SMAX);
    memset(ws->conf_raw, 0, px * sizeof(float));

    if (cost_mode == COST_CENSUS) {
        census(left, left_step, ws->census1, w, h);
        census(right, right_step, ws->census2, w, h);
        census_cost(ws->census1, ws->census2, ws->cost_sad, w, h, D, minD);
    } else {
        bt_grad(left, left_step, ws->grad1, w, h, pfc);
        bt_grad(right, right_step, ws->grad2, w, h, pfc);
        bt_cost(ws->grad1, ws->grad2, left, left_step, right, right_step, ws->cost_sad, w, h, D, minD);
        box_h(ws->cost_sad, ws->cost_acc, w, h, D, bs);
        box_v(ws->cost_acc, ws->cost_sad, w, h, D, bs);
    }

    if (paths >= 2) ss_path_lr(ws->cost_acc, ws->cost_sad, left, left_step, w, h, D, minX1, maxX1, P1, &p2);
    if (paths >= 3) ss_path_tb(ws->cost_acc, ws->cost_sad, left, left_step, w, h, D, P1, &p2);
    ss_path_rl_wta(ws->cost_acc, ws->cost_sad, left, left_step, ws->disp_raw, ws->disp2, ws->disp2_cost,
                   ws->conf_raw, w, h, D, minD, P1, uniq, paths >= 2 ? 1 : 0, &p2);

    if (post & POST_LRCHECK) pseudo_lr_check(ws->disp_raw, ws->disp2, ws->conf_raw, w, h, minD, maxdiff);
    int16_t* fin = ws->disp_raw;
    if (post & POST_MEDIAN) {
        median3x3(ws->disp_raw, ws->disp_med, ws->conf_raw, w, h);
        fin = ws->disp_med;
    }
    if (disp) copy2d(disp, disp_step, fin, (size_t)w * 2, (size_t)w * 2, h);
    if (disp_float && conf_float)
        convert_out(fin, ws->conf_raw, disp_float, df_step, conf_float, cf_step, w, h, invalid);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Params / level geometry / matcher, src/stereo_matcher.cpp:28-338           */
/* ------------------------------------------------------------------------ */
void orc_default_params(orc_params* p)
{
    /* include/pyrsgm/pyrsgm.h:32-82 */
    p->num_disparities = 128; p->min_disparity = 0; p->block_size = 5; p->cost_mode = COST_BT;
    p->p1 = 300; p->p2 = 2400; p->uniqueness_ratio = 10; p->disp12_max_diff = 1;
    p->lr_check = 1; p->median_filter = 1; p->num_paths = 3; p->pre_filter_cap = 63;
    p->pyramid_levels = 0; p->pyramid_coarse_disparities = 128; p->pyramid_max_disparity = 0;
    p->pyramid_min_confidence = 0.05f;
    p->adaptive_p2 = 0; p->p2_alpha = 3.041f; p->p2_beta = 16.137f;
    p->p2_lower_mult = 0.601f; p->p2_upper_mult = 1.77f;
}

static int align16(int v) { return imax(16, ((v + 15) / 16) * 16); }

/* validateParams, src/stereo_matcher.cpp:100-148 */
int orc_validate_params(const orc_params* in, orc_params* out)
{
    orc_params p = *in;
    if (p.num_disparities <= 0 || p.num_disparities > 1024) return -1;
    p.num_disparities = align16(p.num_disparities);
    if (p.num_disparities > 1024) return -1;
    if (p.block_size < 1) return -1;
    p.block_size = imax(3, p.block_size | 1);
    if (p.p1 < 0 || p.p2 < p.p1) return -1;
    if (p.uniqueness_ratio < 0 || p.uniqueness_ratio >= 100) return -1;
    if (p.pre_filter_cap <= 0) return -1;
    p.num_paths = iclamp(p.num_paths, 1, 3);
    if (p.pyramid_levels < 0 || p.pyramid_levels > 4) return -1;
    if (p.pyramid_levels > 0) {
        if (p.min_disparity != 0) return -1;
        if (p.disp12_max_diff < 0) return -1;
        if (p.pyramid_coarse_disparities <= 0) return -1;
        p.pyramid_coarse_disparities = imin(1024, align16(p.pyramid_coarse_disparities));
        if (p.pyramid_max_disparity <= 0) p.pyramid_max_disparity = p.min_disparity + p.num_disparities - 1;
        if (p.pyramid_max_disparity < p.min_disparity) return -1;
        p.pyramid_min_confidence = fminf(fmaxf(p.pyramid_min_confidence, 0.0f), 1.0f);
    }
    if (p.adaptive_p2 && p.p2_beta <= 0.0f) return -1;
    *out = p;
    return 0;
}

/* StereoMatcher::Impl::Impl level geometry, src/stereo_matcher.cpp:169-193 */
int orc_level_geometry(int w, int h, const orc_params* p, orc_level_info* info)
{
    if (w <= 0 || h <= 0) return -1;
    const int levels = p->pyramid_levels;
    int lw = w, lh = h;
    for (int level = 0; level <= levels; ++level) {
        if (level > 0) { lw = (lw + 1) / 2; lh = (lh + 1) / 2; }
        orc_level_info* li = &info[level];
        li->level = level; li->width = lw; li->height = lh;
        if (levels == 0) {
            li->refine = 0;
            li->num_labels = p->num_disparities;
            li->max_disparity = p->min_disparity + p->num_disparities - 1;
            li->block_size = p->block_size;
        } else {
            li->refine = level != levels;
            li->max_disparity = imin(p->pyramid_max_disparity >> level, lw - 1);
            li->num_labels = li->refine ? 16 : align16(imin(p->pyramid_coarse_disparities, li->max_disparity + 1));
            li->block_size = level >= 2 ? 3 : p->block_size;
        }
    }
    return levels + 1;
}

/* StereoMatcher::Impl::postFlags, src/stereo_matcher.cpp:229-236 */
static int post_flags(const orc_params* p, int level)
{
    if (level != 0) return POST_LRCHECK;
    return (p->lr_check ? POST_LRCHECK : 0) | (p->median_filter ? POST_MEDIAN : 0);
}

/* StereoMatcher::Impl::compute, src/stereo_matcher.cpp:238-338 */
int orc_matcher_compute(int w, int h, const orc_params* in,
                        const uint8_t* left, size_t lstep, const uint8_t* right, size_t rstep,
                        int16_t* d16, size_t d16_step, float* d32, size_t d32_step,
                        float* conf, size_t conf_step, const int* lut)
{
    orc_params p;
    if (orc_validate_params(in, &p) != 0 || !left || !right) return -1;
    orc_level_info info[5];
    if (orc_level_geometry(w, h, &p, info) < 0) return -1;
    if (!d16 && !d32 && !conf) return 0;
    const int levels = p.pyramid_levels;
    float* scratch_conf = NULL;
    float* out_conf = conf;
    size_t out_conf_step = conf_step;
    if (!out_conf && d32) {
        scratch_conf = malloc((size_t)w * h * sizeof(float));
        out_conf = scratch_conf;
        out_conf_step = (size_t)w * sizeof(float);
    }
    int ret = 0;
    if (levels == 0) {
        orc_workspace* ws = orc_create_workspace();
        ret = orc_compute_single_scale(ws, left, right, d16, d32, out_conf, lstep, rstep, d16_step,
                                       d32_step, out_conf_step, w, h, p.num_disparities, p.min_disparity,
                                       p.block_size, p.p1, p.p2, p.uniqueness_ratio, p.disp12_max_diff,
                                       p.pre_filter_cap, p.cost_mode, post_flags(&p, 0), p.num_paths,
                                       p.adaptive_p2, p.p2_alpha, p.p2_beta, p.p2_lower_mult,
                                       p.p2_upper_mult, lut);
        orc_destroy_workspace(ws);
        free(scratch_conf);
        return ret;
    }
    uint8_t* pl[5] = {0}; uint8_t* pr[5] = {0};
    int16_t* pd[5] = {0}; float* pc[5] = {0};
    for (int l = 1; l <= levels; ++l) {
        size_t n = (size_t)info[l].width * info[l].height;
        pl[l] = malloc(n); pr[l] = malloc(n); pd[l] = malloc(n * 2); pc[l] = malloc(n * 4);
    }
    const uint8_t* prev_l = left; size_t prev_ls = lstep;
    const uint8_t* prev_r = right; size_t prev_rs = rstep;
    for (int l = 1; l <= levels && ret == 0; ++l) {
        if (orc_pyrdown_u8(prev_l, prev_ls, info[l - 1].width, info[l - 1].height, pl[l], info[l].width,
                           info[l].width, info[l].height) != 0 ||
            orc_pyrdown_u8(prev_r, prev_rs, info[l - 1].width, info[l - 1].height, pr[l], info[l].width,
                           info[l].width, info[l].height) != 0)
            ret = -1;
        prev_l = pl[l]; prev_ls = info[l].width;
        prev_r = pr[l]; prev_rs = info[l].width;
    }
    orc_workspace* ws = orc_create_workspace();
    for (int l = levels; l >= 0 && ret == 0; --l) {
        const orc_level_info* li = &info[l];
        const int refine = li->refine;
        const uint8_t* ll = l == 0 ? left : pl[l];
        const uint8_t* rr = l == 0 ? right : pr[l];
        size_t lls = l == 0 ? lstep : (size_t)li->width;
        size_t rrs = l == 0 ? rstep : (size_t)li->width;
        int16_t* o16 = l == 0 ? d16 : pd[l];
        size_t o16s = l == 0 ? d16_step : (size_t)li->width * 2;
        float* o32 = l == 0 ? d32 : NULL;
        size_t o32s = l == 0 ? d32_step : 0;
        float* oc = l == 0 ? out_conf : pc[l];
        size_t ocs = l == 0 ? out_conf_step : (size_t)li->width * 4;
        const int pw = refine ? info[l + 1].width : 0, ph = refine ? info[l + 1].height : 0;
        ret = orc_compute_level(ws, ll, rr, refine ? pd[l + 1] : NULL, refine ? pc[l + 1] : NULL,
                                o16, o32, oc, lls, rrs, refine ? (size_t)pw * 2 : 0, refine ? (size_t)pw * 4 : 0,
                                o16s, o32s, ocs, li->width, li->height, pw, ph,
                                li->num_labels, p.min_disparity, li->max_disparity, li->block_size,
                                p.p1, p.p2, p.uniqueness_ratio, p.disp12_max_diff, p.pre_filter_cap,
                                p.cost_mode, post_flags(&p, l), p.num_paths, refine,
                                p.pyramid_min_confidence, p.adaptive_p2, p.p2_alpha, p.p2_beta,
                                p.p2_lower_mult, p.p2_upper_mult, lut);
    }
    orc_destroy_workspace(ws);
    for (int l = 1; l <= levels; ++l) { free(pl[l]); free(pr[l]); free(pd[l]); free(pc[l]); }
    free(scratch_conf);
    return ret;
}

/* ---------------------------------------------------------------------------
 * Speckle filter (no counterpart in the reference library): sequential
 * 4-connected flood fill from every unlabelled valid pixel, an explicit
 * stack, then every region of at most max_size pixels set to new_val.
 * ------------------------------------------------------------------------- */
int orc_filter_speckles(int16_t* img, size_t step, int width, int height, int16_t new_val, int max_size,
                        int max_diff)
{
    if (!img || width <= 0 || height <= 0 || max_diff < 0) return -1;
    if (max_size <= 0) return 0;
    const size_t n = (size_t)width * height;
    int* lab = (int*)malloc(n * sizeof(int));
    int* stack = (int*)malloc(n * sizeof(int));
    int* region = (int*)malloc(n * sizeof(int));
    if (!lab || !stack || !region) { free(lab); free(stack); free(region); return -1; }
    for (size_t i = 0; i < n; ++i) lab[i] = -1;
#define PX(x, y) (*(int16_t*)((uint8_t*)img + (size_t)(y) * step + (size_t)(x) * 2))
    for (int y0 = 0; y0 < height; ++y0) {
        for (int x0 = 0; x0 < width; ++x0) {
            const int s = y0 * width + x0;
            if (lab[s] >= 0 || PX(x0, y0) == new_val) continue;
            int top = 0, cnt = 0;
            stack[top++] = s;
            lab[s] = s;
            while (top > 0) {
                const int p = stack[--top];
                region[cnt++] = p;
                const int x = p % width, y = p / width, v = PX(x, y);
                const int nx[4] = {x - 1, x + 1, x, x};
                const int ny[4] = {y, y, y - 1, y + 1};
                for (int k = 0; k < 4; ++k) {
                    if (nx[k] < 0 || nx[k] >= width || ny[k] < 0 || ny[k] >= height) continue;
                    const int q = ny[k] * width + nx[k];
                    const int u = PX(nx[k], ny[k]);
                    if (lab[q] >= 0 || u == new_val || abs(u - v) > max_diff) continue;
                    lab[q] = s;
                    stack[top++] = q;
                }
            }
            if (cnt <= max_size)
                for (int i = 0; i < cnt; ++i) PX(region[i] % width, region[i] / width) = new_val;
        }
    }
#undef PX
    free(lab);
    free(stack);
    free(region);
    return 0;
}
