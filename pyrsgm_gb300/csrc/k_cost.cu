// k_cost.cu -- per-pixel stages of one level: pyrDown, census / BT features,
// refine-label preparation, the adaptive-P2 table and the matching-cost
// volume.  Integer arithmetic, clamps and sentinels follow the reference
// kernels cited at each function (reference file:line).
#include <type_traits>

#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {

constexpr uint32_t kBtBias2 = 0x01000100u;   // 256 in each 16-bit half

// ---------------------------------------------------------------------------
// pyrDown: 5x5 [1 4 6 4 1]^2 / 256, BORDER_REFLECT_101, (sum+128)>>8.
// Reference: src/pyrdown.cu:16-52.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int reflect101(int i, int n)
{
    if (i < 0) i = -i;
    if (i >= n) i = 2 * n - 2 - i;
    return i < 0 ? 0 : i;
}

// One block: 128 x 16 output pixels, a thread per 4 adjacent outputs of a
// row.  The source tile (rows 2*y0 - 2 .. 2*y0 + 32, columns 2*x0 - 4 ..
// 2*x0 + 259, word aligned) is staged as words when it lies inside the
// image and the rows are word aligned, else byte by byte with reflected
// indices.  Each thread sums the five taps of its 11 source columns
// vertically, then the five horizontal taps of each output.
constexpr int kPdX = 128, kPdY = 16;
constexpr int kPdSWB = 2 * kPdX + 8;    // staged source bytes per row
constexpr int kPdSWW = kPdSWB / 4;
constexpr int kPdSH = 2 * kPdY + 3;     // staged source rows

template <int NB>
__global__ void __launch_bounds__(256) k_pyrdown(const __grid_constant__ PyrDownBatch<NB> b)
{
    const PyrDownDesc& P = b.d[blockIdx.z];
    const int x0 = blockIdx.x * kPdX, y0 = blockIdx.y * kPdY;
    if (x0 >= P.dw || y0 >= P.dh) return;
    __shared__ uint32_t tw[kPdSH][kPdSWW];   // byte c of row r: source (reflect(2*y0 - 2 + r), reflect(2*x0 - 4 + c))
    const int sx0 = 2 * x0 - 4, sy0 = 2 * y0 - 2;
    const bool aligned = ((reinterpret_cast<uintptr_t>(P.src) | (uintptr_t)P.sstep) & 3u) == 0;
    if (aligned && sx0 >= 0 && sx0 + kPdSWB <= P.sw && sy0 >= 0 && sy0 + kPdSH <= P.sh) {
        for (int i = threadIdx.x; i < kPdSH * kPdSWW; i += 256) {
            const int r = i / kPdSWW, k = i - r * kPdSWW;
            tw[r][k] = __ldg(reinterpret_cast<const uint32_t*>(P.src + (size_t)(sy0 + r) * P.sstep + sx0) + k);
        }
    } else {
        uint8_t* tb = reinterpret_cast<uint8_t*>(&tw[0][0]);
        for (int i = threadIdx.x; i < kPdSH * kPdSWB; i += 256) {
            const int r = i / kPdSWB, c = i - r * kPdSWB;
            tb[i] = __ldg(P.src + (size_t)reflect101(sy0 + r, P.sh) * P.sstep + reflect101(sx0 + c, P.sw));
        }
    }
    __syncthreads();
    const int tx = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int xb = x0 + 4 * tx;
    if (xb >= P.dw) return;
    const int np = imin(4, P.dw - xb);
#pragma unroll 1
    for (int ty = warp; ty < kPdY; ty += 8) {
        const int y = y0 + ty;
        if (y >= P.dh) break;
        // vertical taps of source columns 2*xb - 2 .. 2*xb + 8 (tile bytes 8*tx + 2 .. 8*tx + 12)
        int v[11];
#pragma unroll
        for (int k = 0; k < 11; ++k) v[k] = 0;
        const int w5[5] = {1, 4, 6, 4, 1};
#pragma unroll
        for (int ky = 0; ky < 5; ++ky) {
            const uint32_t* row = tw[2 * ty + ky] + 2 * tx;
            const uint32_t q0 = row[0], q1 = row[1], q2 = row[2], q3 = row[3];
#pragma unroll
            for (int k = 0; k < 11; ++k) {
                const int bi = k + 2;
                const uint32_t q = bi < 4 ? q0 : bi < 8 ? q1 : bi < 12 ? q2 : q3;
                v[k] += w5[ky] * (int)((q >> (8 * (bi & 3))) & 0xffu);
            }
        }
        uint32_t out = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int sum = v[2 * j] + 4 * v[2 * j + 1] + 6 * v[2 * j + 2] + 4 * v[2 * j + 3] + v[2 * j + 4];
            out |= (uint32_t)((sum + 128) >> 8) << (8 * j);
        }
        uint8_t* dst = P.dst + (size_t)y * P.dstep + xb;
        if (np == 4 && (reinterpret_cast<uintptr_t>(dst) & 3u) == 0) {
            *reinterpret_cast<uint32_t*>(dst) = out;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < np) dst[j] = (uint8_t)(out >> (8 * j));
        }
    }
}

// ---------------------------------------------------------------------------
// Features.  Census: 5x5, replicate borders, MSB first, dy-major, bit =
// neighbour < centre (src/sgm_kernels.cu:251-298).  BT: the Sobel-like
// x-gradient clipped to +-ftzero and offset by ftzero
// (src/sgm_kernels.cu:94-118), plus for both the gradient and intensity
// channels the half-sample interval [lo, hi] of dev_bt_channel_cost
// (src/sgm_kernels.cu:1002-1028) with clamped neighbours.  Census pixels
// store their 25-bit descriptor as one word per pixel; BT pixels store four
// words of 16-bit pairs (gradient low half, intensity high half):
// value + 256, value, lo + 256, hi — the operands of bt_pixel().
//
// The view-0 blocks also start the level: every pixel's disp2 key is
// cleared, and on refine levels the label base is derived from the parent
// level (kernel_PrepareRefineLabels, src/sgm_kernels.cu:955-1000; a
// rejected parent -- invalid disparity or confidence below the minimum --
// becomes kNoParent: every label of the pixel is invalid).
//
// One block: 128 x 16 pixels of one view, a thread per 4 adjacent pixels
// of a row.  The image tile with its 2-pixel border (4 columns on each
// side, so rows stay word aligned) is staged as words when it lies inside
// the image and the rows are word aligned, else byte by byte with
// replicated borders.
// ---------------------------------------------------------------------------
constexpr int kFtX = 128, kFtY = 16;
constexpr int kFtSWB = kFtX + 8;        // staged bytes per row: image columns x0 - 4 .. x0 + 131
constexpr int kFtSWW = kFtSWB / 4;      // ... as words
constexpr int kFtSH = kFtY + 4;         // staged rows: y0 - 2 .. y0 + 17

__device__ __forceinline__ uint32_t byte_of(uint32_t w, int k) { return (w >> (8 * k)) & 0xffu; }

// Label base of pixel x from its parent (the body of
// kernel_PrepareRefineLabels).
__device__ __forceinline__ int16_t refine_base(const LevelDesc& J, int x, int raw, float conf)
{
    const int16_t pinv = (int16_t)((J.minD - 1) * 16);
    if (raw == pinv || conf < J.minConf) return kNoParent;
    const int pred16 = raw * 2;
    const int center = (pred16 + 8) >> 4;
    const int resid = pred16 - center * 16;
    int base = center + (resid < 0 ? -(J.D / 2) : -(J.D / 2) + 1);
    const int physMax = imin(J.maxD, x);
    const int largest = physMax - J.D + 1;
    base = largest >= J.minD ? imin(imax(base, J.minD), largest) : J.minD;
    return (int16_t)base;
}

template <int NJ>
__global__ void __launch_bounds__(256) k_features(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.z >> 1];
    const int view = blockIdx.z & 1;
    const int x0 = blockIdx.x * kFtX, y0 = blockIdx.y * kFtY;
    if (x0 >= J.w || y0 >= J.h) return;
    const uint8_t* img = view ? J.right : J.left;
    const int step = view ? J.rstep : J.lstep;
    uint4* feat = view ? J.featR : J.featL;
    const int W = J.w, H = J.h;

    __shared__ uint32_t tw[kFtSH][kFtSWW];   // byte c of row r: image pixel (y0 - 2 + r, x0 - 4 + c), clamped
    const bool aligned = ((reinterpret_cast<uintptr_t>(img) | (uintptr_t)step) & 3u) == 0;
    if (aligned && x0 >= 4 && x0 + kFtX + 4 <= W && y0 >= 2 && y0 + kFtY + 2 <= H) {
        for (int i = threadIdx.x; i < kFtSH * kFtSWW; i += 256) {
            const int r = i / kFtSWW, k = i - r * kFtSWW;
            tw[r][k] = __ldg(reinterpret_cast<const uint32_t*>(img + (size_t)(y0 - 2 + r) * step + x0 - 4) + k);
        }
    } else {
        uint8_t* tb = reinterpret_cast<uint8_t*>(&tw[0][0]);
        for (int i = threadIdx.x; i < kFtSH * kFtSWB; i += 256) {
            const int r = i / kFtSWB, c = i - r * kFtSWB;
            tb[i] = __ldg(img + (size_t)iclamp(y0 - 2 + r, 0, H - 1) * step + iclamp(x0 - 4 + c, 0, W - 1));
        }
    }
    __syncthreads();
    const int tx = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int xb = x0 + 4 * tx;
    if (xb >= W) return;
    const int np = imin(4, W - xb);                 // pixels of this thread inside the image
    const bool vec = np == 4 && (W & 3) == 0;       // 16-byte stores of 4 words / 8-byte of 4 int16
    const int ftzero = imax(J.pfc, 15) | 1;
#pragma unroll 1
    for (int rr = warp; rr < kFtY; rr += 8) {
        const int y = y0 + rr;
        if (y >= H) break;
        const size_t p = (size_t)y * W + xb;
        if (!PG_IN(p, np, (size_t)W * H, 9)) continue;
        if (J.cost == COST_CENSUS) {
            // bit (dy, dx) of the 4 pixels at once: bytes 2 + dx .. 5 + dx of
            // the 12-byte row window, compared with the 4 centre bytes
            const uint32_t ctr = tw[rr + 2][tx + 1];
            const uint32_t ctr7 = ctr & 0x7f7f7f7fu;
            uint32_t acc[4] = {0u, 0u, 0u, 0u};   // 8 bits per byte lane, first bit highest
            int pos = 0;
#pragma unroll
            for (int dy = 0; dy < 5; ++dy) {
                const uint32_t w0 = tw[rr + dy][tx], w1 = tw[rr + dy][tx + 1], w2 = tw[rr + dy][tx + 2];
                const uint32_t n[5] = {__funnelshift_r(w0, w1, 16), __funnelshift_r(w0, w1, 24), w1,
                                       __funnelshift_r(w1, w2, 8), __funnelshift_r(w1, w2, 16)};
#pragma unroll
                for (int dx = 0; dx < 5; ++dx, ++pos) {
                    // unsigned a < b per byte (SWAR): the low seven bits by a
                    // subtraction that cannot borrow across bytes, then the top bits
                    const uint32_t a = n[dx];
                    const uint32_t d = (a | 0x80808080u) - ctr7;
                    const uint32_t lt = ((~a & ctr) | (~(a ^ ctr) & ~d)) & 0x80808080u;
                    acc[pos >> 3] = (acc[pos >> 3] << 1) | (lt >> 7);
                }
            }
            uint32_t cv[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                cv[j] = (byte_of(acc[0], j) << 17) | (byte_of(acc[1], j) << 9) | (byte_of(acc[2], j) << 1) |
                        byte_of(acc[3], j);
            uint32_t* out = reinterpret_cast<uint32_t*>(feat) + p;
            if (vec) {
                *reinterpret_cast<uint4*>(out) = make_uint4(cv[0], cv[1], cv[2], cv[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j < np) out[j] = cv[j];
            }
        } else {
            // bytes 2 .. 9 of the window rows rr + 1 .. rr + 3: columns xb - 2 .. xb + 5
            uint32_t r1[8], r2[8], r3[8];
            {
                const uint32_t a0 = tw[rr + 1][tx], a1 = tw[rr + 1][tx + 1], a2 = tw[rr + 1][tx + 2];
                const uint32_t b0 = tw[rr + 2][tx], b1 = tw[rr + 2][tx + 1], b2 = tw[rr + 2][tx + 2];
                const uint32_t c0 = tw[rr + 3][tx], c1 = tw[rr + 3][tx + 1], c2 = tw[rr + 3][tx + 2];
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int bi = k + 2;   // byte index in the 12-byte window
                    const uint32_t wa = bi < 4 ? a0 : bi < 8 ? a1 : a2;
                    const uint32_t wb = bi < 4 ? b0 : bi < 8 ? b1 : b2;
                    const uint32_t wc = bi < 4 ? c0 : bi < 8 ? c1 : c2;
                    r1[k] = byte_of(wa, bi & 3);
                    r2[k] = byte_of(wb, bi & 3);
                    r3[k] = byte_of(wc, bi & 3);
                }
            }
            // g[i]: gradient at pixel column xb - 1 + i (window byte k = i + 1)
            int g[6];
#pragma unroll
            for (int i = 0; i < 6; ++i) {
                const int k = i + 1;
                int v = ((int)r2[k + 1] - (int)r2[k - 1]) * 2;
                v += (int)r1[k + 1] - (int)r1[k - 1];
                v += (int)r3[k + 1] - (int)r3[k - 1];
                g[i] = iclamp(v, -ftzero, ftzero) + ftzero;
            }
            auto interval = [](int v, int l, int r, uint32_t& lo, uint32_t& hi) {
                const int vl = (v + l) >> 1, vr = (v + r) >> 1;
                lo = (uint32_t)imin(imin(vl, vr), v);
                hi = (uint32_t)imax(imax(vl, vr), v);
            };
            uint4 f[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                // the neighbour columns are clamped first (x - 1 -> 0 at the left border)
                const int x = xb + j;
                const bool hl = x > 0, hr = x + 1 < W;
                const int gv = g[j + 1], iv = (int)r2[j + 2];
                uint32_t glo, ghi, ilo, ihi;
                interval(gv, hl ? g[j] : gv, hr ? g[j + 2] : gv, glo, ghi);
                interval(iv, hl ? (int)r2[j + 1] : iv, hr ? (int)r2[j + 3] : iv, ilo, ihi);
                const uint32_t X = (uint32_t)gv | ((uint32_t)iv << 16), X0 = glo | (ilo << 16), X1 = ghi | (ihi << 16);
                f[j] = make_uint4(X + kBtBias2, X, X0 + kBtBias2, X1);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (j < np) feat[p + j] = f[j];
        }
        if (view == 0) {
            if (vec) {
                *reinterpret_cast<uint4*>(J.keys + p) = make_uint4(0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j < np) J.keys[p + j] = 0xffffffffu;   // no disp2 candidate yet
            }
            if (J.refine) {
                const int py = imin(y >> 1, J.ph - 1);
                const int16_t* prow = J.pdisp + (size_t)py * J.pd_pitch;
                const float* crow = J.pconf + (size_t)py * J.pc_pitch;
                int16_t b[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int px = imin((xb + j) >> 1, J.pw - 1);
                    b[j] = j < np ? refine_base(J, xb + j, __ldg(prow + px), __ldg(crow + px)) : (int16_t)0;
                }
                int16_t* bo = J.base + p;
                if (vec) {
                    *reinterpret_cast<uint2*>(bo) =
                        make_uint2((uint32_t)(uint16_t)b[0] | ((uint32_t)(uint16_t)b[1] << 16),
                                   (uint32_t)(uint16_t)b[2] | ((uint32_t)(uint16_t)b[3] << 16));
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (j < np) bo[j] = b[j];
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Adaptive P2 table.  dev_adaptive_p2 (src/sgm_kernels.cu:63-74) depends on
// the pixels only through |I(p) - I(p-r)| in [0, 255]; the table holds its
// value for every difference, computed on the device with the same
// expression and the same intrinsic (__expf) so that each entry equals the
// reference's per-voxel value.
// ---------------------------------------------------------------------------
__device__ __noinline__ int adaptive_p2_value(int P2, int cur, int prev, float alpha, float beta,
                                              float lowerMult, float upperMult)
{
    const float diff = fabsf((float)(cur - prev));
    const float ratio = lowerMult + (1.0f + alpha - lowerMult) * __expf(-diff / beta);
    float adaptive = (float)P2 * ratio;
    const float lower = fmaxf(1.0f, (float)P2 * lowerMult);
    const float upper = (float)P2 * upperMult;
    adaptive = fminf(upper, fmaxf(lower, adaptive));
    return (int)(adaptive + 0.5f);
}

__global__ void k_p2_table(int* lut, int P2, float alpha, float beta, float lower, float upper)
{
    const int i = threadIdx.x;
    if (i < 256) lut[i] = adaptive_p2_value(P2, i, 0, alpha, beta, lower, upper);
}

// ---------------------------------------------------------------------------
// Census cost volume.  Coarse / single-scale: kernel_CensusCost
// (src/sgm_kernels.cu:303-327), 24 when x - d - minD is outside the image.
// Refine: kernel_CensusCostLocal (src/sgm_kernels.cu:1112-1133), kMax for a
// geometry-invalid label.  One thread per pixel writes its D labels, eight
// per 16-byte store (label pairs or single labels when D is not a multiple
// of eight).
// ---------------------------------------------------------------------------
template <int NJ>
__global__ void __launch_bounds__(256) k_cost_census(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= J.w || y >= J.h) return;
    const int W = J.w, D = J.D;
    const size_t p = (size_t)y * W + x;
    const uint32_t cl = reinterpret_cast<const uint32_t*>(J.featL)[p];
    const uint32_t* rrow = reinterpret_cast<const uint32_t*>(J.featR) + (size_t)y * W;
    // label d reads right pixel x - off - d when lo <= d <= hi, else `fill`
    int off, lo, hi, fill;
    if (J.refine) {
        off = J.base[p];
        label_range(J, x, off, lo, hi);
        fill = kMax;
    } else {
        off = J.minD;
        lo = imax(0, x - off - (W - 1));
        hi = imin(D - 1, x - off);
        fill = 24;
    }
    auto cost = [&](int d) -> uint32_t {
        return (d >= lo && d <= hi) ? (uint32_t)__popc(cl ^ __ldg(&rrow[x - off - d])) : (uint32_t)fill;
    };
    int16_t* out = J.C + p * D;
    if (!PG_IN(p * D, D, (size_t)W * J.h * D, 10)) return;
    if ((D & 7) == 0) {
        for (int d0 = 0; d0 < D; d0 += 8) {
            uint32_t w[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) w[i] = cost(d0 + 2 * i) | (cost(d0 + 2 * i + 1) << 16);
            reinterpret_cast<uint4*>(out + d0)[0] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    } else {
        for (int d = 0; d < D; ++d) out[d] = (int16_t)cost(d);
    }
}

// BT cost of one (left pixel, right pixel) pair: dev_bt_pixel_cost,
// src/sgm_kernels.cu:1030-1043, i.e. min(255, bt(gradient) + bt(intensity)
// >> 2) with bt(u, v) = min(max(0, u - v.hi, v.lo - u), max(0, v - u.hi,
// u.lo - v)), on both channels at once as 16-bit pairs.  The +256 bias in
// the features keeps every difference positive (no borrow between halves)
// and is the floor of the maxima, subtracted once at the end.
__device__ __forceinline__ int bt_pixel(const uint4 l, const uint4 r)
{
    const uint32_t c0 = __vimax3_u16x2(kBtBias2, l.x - r.w, r.z - l.y);   // 256 + max(0, u - v.hi, v.lo - u)
    const uint32_t c1 = __vimax3_u16x2(kBtBias2, r.x - l.w, l.z - r.y);   // 256 + max(0, v - u.hi, u.lo - v)
    const uint32_t t = __vminu2(c0, c1) - kBtBias2;
    return imin(255, (int)(t & 0xffffu) + (int)(t >> 18));
}

// The same cost plus kBtOff, for the tiled window sums.  With m = min(c0, c1)
// (256 + bt in each half), m >> 18 = 64 + (bt(intensity) >> 2) lies in the
// low half alone, so one __viaddmin_u16x2 adds it to 256 + bt(gradient),
// clamps at 255 + kBtOff and zeroes the high half.  Sums of these carry
// kBtOff per term, taken off once per label.
constexpr uint32_t kBtOff = 320, kBtOffClamp = 255 + kBtOff;
__device__ __forceinline__ uint32_t bt_pixel_off(const uint4 l, const uint4 r)
{
    const uint32_t c0 = __vimax3_u16x2(kBtBias2, l.x - r.w, r.z - l.y);
    const uint32_t c1 = __vimax3_u16x2(kBtBias2, r.x - l.w, l.z - r.y);
    const uint32_t m = __vminu2(c0, c1);
    return __viaddmin_u16x2(m, m >> 18, kBtOffClamp);
}

// ---------------------------------------------------------------------------
// BT coarse / single-scale cost: kernel_BTCost followed by kernel_BoxFilterH
// and kernel_BoxFilterV (src/sgm_kernels.cu:139-239, 354-416), fused.  The
// separable sums keep the reference's two saturation points:
//   C = min(MAX, sum_dy min(MAX, sum_dx bt(clamp(y+dy), clamp(x+dx), d))).
// One block: 32 x 8 output pixels x 16 labels.  bt values are staged in
// shared memory for the (8+2h) x (32+2h) window of clamped pixels.
// ---------------------------------------------------------------------------
constexpr int kBxX = 32, kBxY = 8, kBxD = 16;

template <int NJ>
__global__ void __launch_bounds__(256) k_cost_bt_box(const __grid_constant__ Jobs<NJ> jobs, int maxHalf, int nxt)
{
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x0 = (blockIdx.x % nxt) * kBxX;
    const int d0 = (blockIdx.x / nxt) * kBxD;
    const int y0 = blockIdx.y * kBxY;
    if (x0 >= J.w || y0 >= J.h || d0 >= J.D) return;
    const int h = J.bs / 2;
    const int SW = kBxX + 2 * maxHalf, SH = kBxY + 2 * maxHalf;
    extern __shared__ unsigned char sm[];
    uint8_t* bt = sm;                                               // [SH][SW][kBxD]
    uint16_t* hs = reinterpret_cast<uint16_t*>(sm + ((SH * SW * kBxD + 15) & ~15));  // [SH][kBxX][kBxD]
    const int W = J.w, H = J.h;
    const int sw = kBxX + 2 * h, sh = kBxY + 2 * h;
    for (int i = threadIdx.x; i < sh * sw * kBxD; i += blockDim.x) {
        const int dd = i % kBxD;
        const int j = (i / kBxD) % sw;
        const int r = i / (kBxD * sw);
        const int gy = iclamp(y0 - h + r, 0, H - 1), gx = iclamp(x0 - h + j, 0, W - 1);
        const int x2 = gx - (d0 + dd + J.minD);
        int v = 255;
        if (x2 >= 0 && x2 < W) v = bt_pixel(J.featL[(size_t)gy * W + gx], J.featR[(size_t)gy * W + x2]);
        bt[(r * SW + j) * kBxD + dd] = (uint8_t)v;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < sh * kBxX * kBxD; i += blockDim.x) {
        const int dd = i % kBxD;
        const int j = (i / kBxD) % kBxX;
        const int r = i / (kBxD * kBxX);
        int s = 0;
        for (int k = 0; k <= 2 * h; ++k) s += bt[(r * SW + j + k) * kBxD + dd];
        hs[(r * kBxX + j) * kBxD + dd] = (uint16_t)imin(kMax, s);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBxY * kBxX * (kBxD / 2); i += blockDim.x) {
        const int dp = i % (kBxD / 2);
        const int j = (i / (kBxD / 2)) % kBxX;
        const int r = i / ((kBxD / 2) * kBxX);
        const int x = x0 + j, y = y0 + r;
        if (x >= W || y >= H) continue;
        int s0 = 0, s1 = 0;
        for (int k = 0; k <= 2 * h; ++k) {
            s0 += hs[((r + k) * kBxX + j) * kBxD + 2 * dp];
            s1 += hs[((r + k) * kBxX + j) * kBxD + 2 * dp + 1];
        }
        const uint32_t v = (uint32_t)imin(kMax, s0) | ((uint32_t)imin(kMax, s1) << 16);
        reinterpret_cast<uint32_t*>(J.C + ((size_t)y * W + x) * J.D + d0)[dp] = v;
    }
}

// ---------------------------------------------------------------------------
// BT refine cost: kernel_BTWindowCostLocal, src/sgm_kernels.cu:1075-1110.
// For label d of pixel p the reference sums, over the blockSize^2 window of
// clamped pixels q, the BT cost of q at the real disparity base_p + d (255
// when q - (base_p + d) leaves the image), clamps the sum to kMax - 1, and
// writes kMax for a geometry-invalid label.  The sum depends on p only
// through the window and the real disparity, so one 32x16 tile evaluates
// each (window pixel, real disparity) pair once when the real disparities
// its pixels need, [min base, max base + D - 1], span at most kTiRn:
//   staging: the features of every window row of the tile (left: one per
//            window column, clamped; right: the ones its disparities reach)
//            are copied once into shared memory with cp.async;
//   phase 1: the (window row, two adjacent real disparities) units of a
//            half row of 16 output columns are numbered row-major and cut
//            into groups of 32, one unit per lane, dealt to the 8 warps in
//            turn; a lane walks its half row left to right and keeps the
//            running sums of the last blockSize costs of both disparities
//            (sums along x, into shared memory), loading each left and
//            right feature once for the two.  A tile usually needs 17 real
//            disparities, so numbering the units this way keeps nearly
//            every lane busy;
//   phase 2: a thread per pixel adds blockSize rows of those sums, two
//            labels per 32-bit add, from its own real-disparity offset.
// Window sums are exact integers (at most 25 * 255 here, no intermediate
// clamp in the reference); the terms carry kBtOff each (bt_pixel_off), at
// most 25 * 575 per 16-bit half, removed after the column sums.  Tiles
// whose parents disagree more widely are
// split into two base clusters (a pass each); pixels in neither, or a
// wider window, evaluate each window directly.
// ---------------------------------------------------------------------------
constexpr int kTiX = 32, kTiY = 16, kTiRn = 32, kTiMaxHalf = 2;
constexpr int kTiWarps = 8;
constexpr int kTiSeg = 16;                          // output columns of a half row
constexpr int kTiRows = kTiY + 2 * kTiMaxHalf;      // window rows at most
constexpr int kTiRs = kTiRn + 2;   // halves per (row, column): 17 words, odd, so columns hit distinct banks
constexpr int kTiSL = kTiX + 2 * kTiMaxHalf;        // staged left features per window row
constexpr int kTiSR = kTiSL + kTiRn - 1;            // staged right features per window row
constexpr size_t kTiHs = (size_t)kTiRows * kTiX * kTiRs * 2;
constexpr size_t kTiSmem = kTiHs + (size_t)kTiRows * (kTiSL + kTiSR) * 16;

__device__ __forceinline__ void tile_cp16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void tile_commit_wait()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// Sums along x, for a cluster of real disparities rmin .. rmin + rn - 1,
// of every window row of the tile (see above).
template <int HW>
__device__ __forceinline__ void bt_row_sums(const LevelDesc& J, uint16_t* hs, uint4* st, int x0, int y0, int rmin,
                                            int rn, int warp, int lane)
{
    constexpr int R = kTiY + 2 * HW;     // window rows
    constexpr int SW = kTiSeg + 2 * HW;  // window columns of a half row
    const int W = J.w, H = J.h;
    uint4* sl = st;                      // [R][kTiSL]  left, columns x0 - HW + j (clamped)
    uint4* sr = st + kTiRows * kTiSL;    // [R][kTiSR]  right, columns xrs + k (inside the image only)
    const int xrs = x0 - HW - (rmin + rn - 1);
    const int nsl = kTiX + 2 * HW, nsr = nsl + rn - 1;
    // staging (the block's threads, one pass of copies)
    for (int i = threadIdx.x; i < R * nsl; i += blockDim.x) {
        const int r = i / nsl, j = i - r * nsl;
        const int gy = iclamp(y0 - HW + r, 0, H - 1);
        tile_cp16(sl + r * kTiSL + j, J.featL + (size_t)gy * W + iclamp(x0 - HW + j, 0, W - 1));
    }
    for (int i = threadIdx.x; i < R * nsr; i += blockDim.x) {
        const int r = i / nsr, k = i - r * nsr;
        const int gy = iclamp(y0 - HW + r, 0, H - 1);
        const int xx = xrs + k;
        if (xx >= 0 && xx < W) tile_cp16(sr + r * kTiSR + k, J.featR + (size_t)gy * W + xx);
    }
    tile_commit_wait();
    __syncthreads();
    // every window column of the tile inside the image, and every right pixel too
    const bool interior = x0 - HW >= 0 && x0 + kTiX - 1 + HW < W && xrs >= 0 && xrs + nsr - 1 < W;
    // Units: (window row, real-disparity pair ri, ri + 1) of a half row,
    // numbered row-major, one per lane.  Real disparity ri + 1 needs at
    // window column j the right feature that ri needed at column j - 1, so
    // a lane loads one left and one right feature per column for two sums
    // and stores both as one word.  With rn odd the last pair's second
    // half is past the cluster: computed, never read.
    const int rp = (rn + 1) >> 1;
    const int pairs = R * rp;
    const int chunks = (pairs + 31) >> 5;
    for (int u = warp; u < 2 * chunks; u += kTiWarps) {
        const int seg = u & 1, f = (u >> 1) * 32 + lane;
        const bool on = f < pairs;
        const int fr = on ? f : pairs - 1;
        const int row = fr / rp, ri = 2 * (fr - row * rp);
        const int real = rmin + ri;
        const int c0 = seg * kTiSeg;               // first window column of the half row (tile-relative)
        const uint4* lrow = sl + row * kTiSL + c0;
        const uint4* rrow = sr + row * kTiSR;
        uint32_t* out = reinterpret_cast<uint32_t*>(hs + ((size_t)row * kTiX + c0) * kTiRs + ri);
        auto walk = [&](auto inner) {
            constexpr bool IN = decltype(inner)::value;
            // right feature of window column j for ri: srl[j]; for ri + 1: srl[j - 1] (interior)
            const uint4* srl = rrow + c0 - ri + rn - 1;
            uint4 rprev = IN ? srl[-1] : make_uint4(0u, 0u, 0u, 0u);
            uint32_t q0[2 * HW + 1], q1[2 * HW + 1];
#pragma unroll
            for (int i = 0; i < 2 * HW + 1; ++i) q0[i] = q1[i] = 0;
            uint32_t s0 = 0, s1 = 0;
#pragma unroll
            for (int j = 0; j < SW; ++j) {
                uint32_t e0, e1;   // costs + kBtOff at real disparities ri, ri + 1
                if (IN) {
                    const uint4 l = lrow[j], r = srl[j];
                    e0 = bt_pixel_off(l, r);
                    e1 = bt_pixel_off(l, rprev);
                    rprev = r;
                } else {
                    const int gx = iclamp(x0 - HW + c0 + j, 0, W - 1);
                    const int x2 = gx - real, x3 = x2 - 1;
                    const uint4 l = lrow[j];
                    e0 = (x2 >= 0 && x2 < W) ? bt_pixel_off(l, rrow[x2 - xrs]) : kBtOffClamp;
                    e1 = (x3 >= 0 && x3 < W) ? bt_pixel_off(l, rrow[x3 - xrs]) : kBtOffClamp;
                }
                s0 += e0;
                s1 += e1;
                if (j >= 2 * HW && on) out[(j - 2 * HW) * (kTiRs / 2)] = s0 | (s1 << 16);
                if (HW > 0) {
                    s0 -= q0[0];
                    s1 -= q1[0];
#pragma unroll
                    for (int i = 0; i + 1 < 2 * HW; ++i) {
                        q0[i] = q0[i + 1];
                        q1[i] = q1[i + 1];
                    }
                    q0[2 * HW - 1 < 0 ? 0 : 2 * HW - 1] = e0;
                    q1[2 * HW - 1 < 0 ? 0 : 2 * HW - 1] = e1;
                } else {
                    s0 = s1 = 0;
                }
            }
        };
        if (interior) walk(std::true_type{});
        else walk(std::false_type{});
    }
}

template <int NJ>
__global__ void __launch_bounds__(256, 3) k_cost_bt_tiled(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x0 = blockIdx.x * kTiX, y0 = blockIdx.y * kTiY;
    if (x0 >= J.w || y0 >= J.h) return;
    const int W = J.w, H = J.h, D = J.D, h = J.bs / 2;
    extern __shared__ __align__(16) uint16_t hs[];   // [kTiRows][kTiX][kTiRs], then the staged features
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint4* stg = reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(hs) + kTiHs);
    __shared__ int wred[2][kTiWarps];
    // a thread's two pixels: (x0 + lane, y0 + warp) and (x0 + lane, y0 + warp + 8)
    const int x = x0 + lane;
    int yq[2], bq[2];
    bool inq[2], hasq[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        yq[i] = y0 + warp + 8 * i;
        inq[i] = x < W && yq[i] < H;
        bq[i] = inq[i] ? (int)J.base[(size_t)yq[i] * W + x] : (int)kNoParent;
        hasq[i] = inq[i] && bq[i] != kNoParent;
    }
    auto block_minmax = [&](bool in0, bool in1, int& mn, int& mx) {
        const int a = __reduce_min_sync(0xffffffffu, imin(in0 ? bq[0] : INT_MAX, in1 ? bq[1] : INT_MAX));
        const int z = __reduce_max_sync(0xffffffffu, imax(in0 ? bq[0] : INT_MIN, in1 ? bq[1] : INT_MIN));
        __syncthreads();   // wred reused
        if (lane == 0) { wred[0][warp] = a; wred[1][warp] = z; }
        __syncthreads();
        mn = INT_MAX;
        mx = INT_MIN;
#pragma unroll
        for (int i = 0; i < kTiWarps; ++i) { mn = imin(mn, wred[0][i]); mx = imax(mx, wred[1][i]); }
    };
    // Real disparities the tile needs: [min base, max base + D - 1].  When
    // they span more than kTiRn (a depth edge through the tile), the bases
    // are split at the midpoint of their range into two clusters, each
    // handled by its own pass when it fits.
    int bmin, bmax;
    block_minmax(hasq[0], hasq[1], bmin, bmax);
    int ncl = 0, cut = INT_MAX;
    int cmin[2] = {bmin, 0}, cmax[2] = {bmax, 0};
    if (bmax != INT_MIN && h <= kTiMaxHalf) {
        if (bmax + D - bmin <= kTiRn) {
            ncl = 1;
        } else {
            cut = bmin + ((bmax - bmin) >> 1);
            int a0, a1, b0, b1;
            block_minmax(hasq[0] && bq[0] <= cut, hasq[1] && bq[1] <= cut, a0, a1);
            block_minmax(hasq[0] && bq[0] > cut, hasq[1] && bq[1] > cut, b0, b1);
            if (a1 + D - a0 <= kTiRn && b1 + D - b0 <= kTiRn) {
                ncl = 2;
                cmin[0] = a0; cmax[0] = a1; cmin[1] = b0; cmax[1] = b1;
            }
        }
    }
    const bool vec = (D & 7) == 0;
    for (int c = 0; c < ncl; ++c) {
        const int rmin = cmin[c], rn = cmax[c] + D - cmin[c];
        if (h == 2) bt_row_sums<2>(J, hs, stg, x0, y0, rmin, rn, warp, lane);
        else if (h == 1) bt_row_sums<1>(J, hs, stg, x0, y0, rmin, rn, warp, lane);
        else bt_row_sums<0>(J, hs, stg, x0, y0, rmin, rn, warp, lane);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            if (!(hasq[i] && (ncl == 1 || (c == 0) == (bq[i] <= cut)))) continue;
            const int ty = warp + 8 * i;
            if (!PG_IN(((size_t)yq[i] * W + x) * D, D, (size_t)W * H * D, 11)) continue;
            int lo, hi;
            label_range(J, x, bq[i], lo, hi);
            int16_t* out = J.C + ((size_t)yq[i] * W + x) * D;
            // packed pair sums of 2h+1 rows from offset ri0 = b - rmin (halves), 8 labels per chunk;
            // each half carries kBtOff per window pixel
            const int ri0 = bq[i] - rmin;
            const uint32_t sh = (uint32_t)(ri0 & 1) * 16;
            const uint32_t off2 = (kBtOff * (uint32_t)((2 * h + 1) * (2 * h + 1))) * 0x10001u;
            for (int d0 = 0; d0 < D; d0 += 8) {
                uint32_t acc[5] = {0u, 0u, 0u, 0u, 0u};
                for (int k = 0; k <= 2 * h; ++k) {
                    const uint32_t* row =
                        reinterpret_cast<const uint32_t*>(hs + ((ty + k) * kTiX + lane) * kTiRs) + ((ri0 + d0) >> 1);
#pragma unroll
                    for (int j = 0; j < 5; ++j) acc[j] += row[j];
                }
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    w[q] = __funnelshift_r(acc[q], acc[q + 1], sh) - off2;
                    const int d = d0 + 2 * q;
                    if (d < lo || d > hi) w[q] = (w[q] & 0xffff0000u) | (uint32_t)kMax;
                    if (d + 1 < lo || d + 1 > hi) w[q] = (w[q] & 0xffffu) | ((uint32_t)kMax << 16);
                }
                if (vec) {
                    reinterpret_cast<uint4*>(out + d0)[0] = make_uint4(w[0], w[1], w[2], w[3]);
                } else {
                    for (int q = 0; q < 8 && d0 + q < D; ++q)
                        out[d0 + q] = (int16_t)((w[q >> 1] >> ((q & 1) * 16)) & 0xffffu);
                }
            }
        }
        __syncthreads();   // the next cluster's row sums overwrite hs
    }
    // direct window per pixel (no parent, or not in a cluster)
#pragma unroll 1
    for (int i = 0; i < 2; ++i) {
        const bool in = i ? inq[1] : inq[0], has = i ? hasq[1] : hasq[0];
        if (!in || (ncl > 0 && has)) continue;
        const int y = i ? yq[1] : yq[0], b = i ? bq[1] : bq[0];
        int lo, hi;
        label_range(J, x, b, lo, hi);
        int16_t* out = J.C + ((size_t)y * W + x) * D;
        for (int d0 = 0; d0 < D; d0 += 8) {
            int sum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (b != kNoParent) {
                for (int dy = -h; dy <= h; ++dy) {
                    const int gy = iclamp(y + dy, 0, H - 1);
                    const uint4* lrow = J.featL + (size_t)gy * W;
                    const uint4* rrow = J.featR + (size_t)gy * W;
                    for (int dx = -h; dx <= h; ++dx) {
                        const int gx = iclamp(x + dx, 0, W - 1);
                        const uint4 lf = __ldg(&lrow[gx]);
#pragma unroll
                        for (int q = 0; q < 8; ++q) {
                            const int x2 = gx - (b + d0 + q);
                            sum[q] += (x2 >= 0 && x2 < W) ? bt_pixel(lf, __ldg(&rrow[x2])) : 255;
                        }
                    }
                }
            }
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int d = d0 + 2 * q;
                const uint32_t v0 = (d >= lo && d <= hi) ? (uint32_t)imin(sum[2 * q], kMax - 1) : (uint32_t)kMax;
                const uint32_t v1 =
                    (d + 1 >= lo && d + 1 <= hi) ? (uint32_t)imin(sum[2 * q + 1], kMax - 1) : (uint32_t)kMax;
                w[q] = v0 | (v1 << 16);
            }
            if (vec) {
                reinterpret_cast<uint4*>(out + d0)[0] = make_uint4(w[0], w[1], w[2], w[3]);
            } else {
                for (int q = 0; q < 8 && d0 + q < D; ++q) out[d0 + q] = (int16_t)((w[q >> 1] >> ((q & 1) * 16)) & 0xffffu);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int NB>
cudaError_t launch_pyrdown(const PyrDownBatch<NB>& b, int max_dw, int max_dh, cudaStream_t st)
{
    dim3 grid((max_dw + kPdX - 1) / kPdX, (max_dh + kPdY - 1) / kPdY, b.n);
    prof_begin(st);
    k_pyrdown<NB><<<grid, 256, 0, st>>>(b);
    count_launch();
    if (prof_enabled()) {
        double by = 0;
        for (int i = 0; i < b.n; ++i) by += (double)b.d[i].sw * b.d[i].sh + (double)b.d[i].dw * b.d[i].dh;
        prof_end(PK_PYRDOWN, by, st);
    }
    return launched(st, "k_pyrdown");
}
template cudaError_t launch_pyrdown<1>(const PyrDownBatch<1>&, int, int, cudaStream_t);
template cudaError_t launch_pyrdown<2>(const PyrDownBatch<2>&, int, int, cudaStream_t);
template cudaError_t launch_pyrdown<kBatchPyr>(const PyrDownBatch<kBatchPyr>&, int, int, cudaStream_t);

cudaError_t launch_p2_table(int* lut, int P2, float alpha, float beta, float lower, float upper, cudaStream_t st)
{
    prof_begin(st);
    k_p2_table<<<1, 256, 0, st>>>(lut, P2, alpha, beta, lower, upper);
    count_launch();
    prof_end(PK_P2TABLE, 1024.0, st);
    return launched(st, "k_p2_table");
}

template <int NJ>
cudaError_t launch_prepare(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    dim3 gf((e.max_w + kFtX - 1) / kFtX, (e.max_h + kFtY - 1) / kFtY, 2 * jobs.n);
    prof_begin(st);
    k_features<NJ><<<gf, 256, 0, st>>>(jobs);
    count_launch();
    if (prof_enabled()) {
        // read u8 and write features of both views, write the keys; refine
        // levels read the quarter-size parent and write the label base
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double px = (double)d.w * d.h;
            by += px * (2 * (1 + (d.cost == COST_CENSUS ? 4 : 16)) + 4 + (d.refine ? 2 + 6.0 / 4 : 0));
        }
        prof_end(PK_FEATURES, by, st);
    }
    return launched(st, "k_features");
}

// All jobs in `jobs` share the cost mode and the refine flag.
template <int NJ>
cudaError_t launch_cost(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    const LevelDesc& J0 = jobs.d[0];
    prof_begin(st);
    if (J0.cost == COST_CENSUS) {
        dim3 g((e.max_w + 31) / 32, (e.max_h + 7) / 8, jobs.n);
        k_cost_census<NJ><<<g, 256, 0, st>>>(jobs);
    } else if (J0.refine) {
        cudaError_t err = cudaFuncSetAttribute(k_cost_bt_tiled<NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)kTiSmem);
        if (err != cudaSuccess) return err;
        dim3 g((e.max_w + kTiX - 1) / kTiX, (e.max_h + kTiY - 1) / kTiY, jobs.n);
        k_cost_bt_tiled<NJ><<<g, 256, kTiSmem, st>>>(jobs);
    } else {
        int maxHalf = 0;
        for (int j = 0; j < jobs.n; ++j) maxHalf = std::max(maxHalf, jobs.d[j].bs / 2);
        const int SW = kBxX + 2 * maxHalf, SH = kBxY + 2 * maxHalf;
        const size_t smem = ((SH * SW * kBxD + 15) & ~15) + (size_t)SH * kBxX * kBxD * 2;
        if (smem > 48 * 1024) {
            cudaError_t err = cudaFuncSetAttribute(k_cost_bt_box<NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem);
            if (err != cudaSuccess) return err;
        }
        const int nxt = (e.max_w + kBxX - 1) / kBxX;
        dim3 g(nxt * ((e.max_D + kBxD - 1) / kBxD), (e.max_h + kBxY - 1) / kBxY, jobs.n);
        k_cost_bt_box<NJ><<<g, 256, smem, st>>>(jobs, maxHalf, nxt);
    }
    count_launch();
    // write the int16 volume, read both views' features (and the label base)
    prof_end(PK_COST, jobs_vox(jobs) * 2 + jobs_px(jobs) * ((J0.cost == COST_CENSUS ? 8 : 32) + (J0.refine ? 2 : 0)), st);
    return launched(st, J0.cost == COST_CENSUS ? "k_cost_census" : J0.refine ? "k_cost_bt_tiled" : "k_cost_bt_box");
}

#define PG_INST(NJ)                                                                          \
    template cudaError_t launch_prepare<NJ>(const Jobs<NJ>&, const LevelExtent&, cudaStream_t); \
    template cudaError_t launch_cost<NJ>(const Jobs<NJ>&, const LevelExtent&, cudaStream_t);
PG_INST(1)
PG_INST(kBatchJobs)
#undef PG_INST

}  // namespace pg
