// k_paths_packed.cuh -- path aggregation for D = 8*T labels (16, 32, 64):
// the labels of one path chain are packed two per 32-bit word and spread
// over a group of T adjacent threads, four words (eight labels) each.
//
// The recurrence of a step (reference: src/sgm_kernels.cu:560-565
// single-scale, 1230-1252 pyramid) runs on 16-bit pairs with the DPX
// integer instructions:
//   best = min(L[s], min(L[s-1] + P1, lj), L[s+1] + P1)  __viaddmin / __vimin3
//   v    = min(c + (best - minPrev), SHRT_MAX)           __viaddmin
// where s is the label of the previous pixel with the same real disparity
// (pyramid levels shift labels by base - prevBase), lj = min(SHRT_MAX,
// minPrev + P2).  No lane of these can wrap: every operand is at most
// SHRT_MAX, P1 is clamped to 0x8000, best <= lj <= SHRT_MAX and best >=
// minPrev, so a plain 32-bit add/subtract never carries between halves.
//
// Pyramid rules without per-label masks:
//   * labels outside label_range have cost SHRT_MAX in refine volumes (the
//     cost kernels write it) and are forced to it at coarse-level borders;
//     min(SHRT_MAX + x, SHRT_MAX) keeps them at SHRT_MAX;
//   * a chain is inactive exactly when minPrev == SHRT_MAX, and then every
//     previous label is SHRT_MAX, so best - minPrev == 0 and v = c;
//   * an active chain whose best is SHRT_MAX gives SHRT_MAX (the sign of
//     best + 1 per half, replicated by prmt).
//
// Each step a thread stores its four words of the previous step into a
// guard-padded shared buffer of its chain (double-buffered, one __syncwarp
// per step) and reads back the six words of its shifted window; chain
// minima and WTA argmins reduce over the group by __shfl_xor_sync.  The
// buffers are placed so that the 32 threads of a warp touch 32 different
// banks whenever the chains share their label shift.
//
// Horizontal pass: a warp holds 16/T rows, each with an L->R group and an
// R->L group walking towards each other; the first chain at a pixel leaves
// its partial sum (with the top->bottom costs) in V, or in a shared-memory
// band near the meeting point, the second finishes the pixel (deferred WTA).
// The disp2 candidates go to the per-pixel keys with atomicMin; the LR check
// reads them in the post kernel.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {
namespace pk {

constexpr uint32_t kMax2 = 0x7fff7fffu;
constexpr uint32_t kOne2 = 0x00010001u;
constexpr int kPF = 4;      // register prefetch distance in steps
constexpr int kWarps = 4;   // warps per block

__device__ __forceinline__ uint32_t dup(int v) { return ((uint32_t)v & 0xffffu) * 0x10001u; }

// 0xffff in each 16-bit half whose bit 15 is set, else 0.
__device__ __forceinline__ uint32_t sign_mask2(uint32_t x)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, 0xBB99;" : "=r"(r) : "r"(x));
    return r;
}

template <int T>
struct Grp {
    static constexpr int D = 8 * T;             // labels per chain
    static constexpr int CPW = 32 / T;          // chains per warp
    static constexpr int PADW = D / 2 + 1;      // guard words before label 0 (D + 2 halves)
    static constexpr int LENW = PADW + D + 2;   // words a shifted window can touch
    static constexpr int GPB = 8 / T;           // chains per 32-bank row of the layout
    static constexpr int NEED = LENW + 35 - 4 * T;
    static constexpr int CS = (NEED + 31) / 32 * 32;   // chain stride (words, multiple of 32)
    static constexpr int BUFW = CPW * CS;              // one buffer of a warp
    // Word offset of chain c's buffer: c * CS plus a bank offset so that
    // word j of thread k of chain c lands in bank off(c) + 4k + j (mod 32),
    // distinct over the warp.
    __device__ static int off(int c) { return c * CS + 4 * T * (c % GPB) + c / GPB; }
};

template <int T>
struct GChain {
    uint32_t L[4];
    int mp;        // minimum of the previous step over the chain's labels
    int prevBase;
};

template <int T>
__device__ __forceinline__ void gchain_init(GChain<T>& s, int minD)
{
#pragma unroll
    for (int i = 0; i < 4; ++i) s.L[i] = kMax2;
    s.mp = 0x7fff;
    s.prevBase = minD;
}

// One step of the chain: c = this thread's eight costs of the pixel,
// buf = the chain's buffer of this step's parity.
template <int T, bool PYR>
__device__ __forceinline__ void gstep(GChain<T>& s, const uint32_t (&c)[4], int base, int p2, uint32_t p12,
                                      uint32_t* buf, int k)
{
    using G = Grp<T>;
    constexpr int D = G::D;
#pragma unroll
    for (int i = 0; i < 4; ++i) buf[G::PADW + 4 * k + i] = s.L[i];
    __syncwarp();
    int delta = PYR ? base - s.prevBase : 0;
    delta = iclamp(delta, -(D + 1), D + 1);
    const int i0 = 2 * G::PADW + delta - 1 + 8 * k;    // half index of label (8k - 1) after the shift
    const uint32_t* wp = buf + (i0 >> 1);
    const uint32_t sh = (uint32_t)(i0 & 1) * 16;
    uint32_t w0[6];
#pragma unroll
    for (int j = 0; j < 6; ++j) w0[j] = wp[j];
    uint32_t w[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) w[j] = __funnelshift_r(w0[j], w0[j + 1], sh);
    const int lj = imin(0x7fff, s.mp + p2);
    const uint32_t lj2 = dup(lj), mp2 = dup(s.mp);
    const uint32_t inc2 = (PYR && s.mp < 0x7fff) ? kOne2 : 0u;
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        const uint32_t n0 = __funnelshift_r(w[m], w[m + 1], 16);   // (L[s], L[s+1])
        const uint32_t t = __viaddmin_u16x2(w[m], p12, lj2);       // min(L[s-1] + P1, lj)
        const uint32_t best = __vimin3_u16x2(n0, t, w[m + 1] + p12);
        uint32_t v = __viaddmin_u16x2(c[m], best - mp2, kMax2);
        if constexpr (PYR) v |= sign_mask2(best + inc2) & kMax2;
        s.L[m] = v;
    }
    uint32_t m2 = __vminu2(__vimin3_u16x2(s.L[0], s.L[1], s.L[2]), s.L[3]);
#pragma unroll
    for (int o = 1; o < T; o <<= 1) m2 = __vminu2(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    s.mp = imin((int)(m2 & 0xffffu), (int)(m2 >> 16));
    s.prevBase = base;
}

// Coarse pyramid levels: labels outside label_range take SHRT_MAX.
template <int T>
__device__ __forceinline__ void mask_labels(uint32_t (&c)[4], int lo, int hi, int k)
{
    if (lo <= 8 * k && hi >= 8 * k + 7) return;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int d0 = 8 * k + 2 * i;
        const bool ok0 = d0 >= lo && d0 <= hi, ok1 = d0 + 1 >= lo && d0 + 1 <= hi;
        c[i] |= (ok0 ? 0u : 0x7fffu) | (ok1 ? 0u : 0x7fff0000u);
    }
}

// Partial sum of the first path at a pixel and total at the second.
template <bool PYR>
__device__ __forceinline__ uint32_t gcombine(uint32_t a, uint32_t b)
{
    if constexpr (PYR) {
        // saturate at SHRT_MAX - 1; SHRT_MAX when either side is SHRT_MAX
        const uint32_t s = __viaddmin_u16x2(a, b, 0x7ffe7ffeu);
        return s | (sign_mask2((a + kOne2) | (b + kOne2)) & kMax2);
    } else {
        return __viaddmin_u16x2(a, b, kMax2);
    }
}

__device__ __forceinline__ void to4(const uint4 q, uint32_t (&v)[4])
{
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
__device__ __forceinline__ uint4 from4(const uint32_t (&v)[4]) { return make_uint4(v[0], v[1], v[2], v[3]); }

// Winner-take-all of one pixel over a chain group (kernel_WTA_Subpixel,
// src/sgm_kernels.cu:573-640; pyramid kernel_PyramidWTA,
// src/sgm_kernels.cu:1290-1370).  Every lane of the warp calls it; `doit`
// gates the writes.  scr: this warp's 128-word scratch.
template <int T, bool PYR>
__device__ __forceinline__ void gwta(const LevelDesc& J, bool doit, int y, int x, const uint32_t (&tot)[4], int base,
                                     uint32_t* scr, int lane, int k)
{
    constexpr int D = 8 * T;
    // first label of the minimum: per thread, then over the group (cost << 16 | label)
    const uint32_t m2 = __vminu2(__vimin3_u16x2(tot[0], tot[1], tot[2]), tot[3]);
    const int lmin = imin((int)(m2 & 0xffffu), (int)(m2 >> 16));
    const uint32_t mc2 = dup(lmin);
    int li = 7;
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        const uint32_t e = tot[i] - mc2;                       // zero half where equal (no borrow)
        const uint32_t z = (e - kOne2) & ~e & 0x80008000u;     // lowest set bit marks the first zero half
        if (z) li = 2 * i + ((z & 0x8000u) ? 0 : 1);
    }
    unsigned key = ((unsigned)lmin << 16) | (unsigned)(8 * k + li);
#pragma unroll
    for (int o = 1; o < T; o <<= 1) key = umin(key, __shfl_xor_sync(0xffffffffu, key, o));
    const int minCost = (int)(key >> 16), bestD = (int)(key & 0xffffu);
    // neighbours of the best label, then the minimum over |d - best| > 1
    reinterpret_cast<uint4*>(scr)[lane] = from4(tot);
    __syncwarp();
    int16_t* lab = reinterpret_cast<int16_t*>(scr) + (lane - k) * 8;
    const bool owner = (bestD >> 3) == k;
    int c0 = 0, c1 = 0, c2 = 0;
    if (owner) {
        c1 = lab[bestD];
        if (bestD > 0) { c0 = lab[bestD - 1]; lab[bestD - 1] = 0x7fff; }
        if (bestD + 1 < D) { c2 = lab[bestD + 1]; lab[bestD + 1] = 0x7fff; }
        lab[bestD] = 0x7fff;
    }
    __syncwarp();
    uint32_t q[4];
    to4(reinterpret_cast<const uint4*>(scr)[lane], q);
    const uint32_t a2 = __vminu2(__vimin3_u16x2(q[0], q[1], q[2]), q[3]);
    int alt = imin((int)(a2 & 0xffffu), (int)(a2 >> 16));
#pragma unroll
    for (int o = 1; o < T; o <<= 1) alt = imin(alt, __shfl_xor_sync(0xffffffffu, alt, o));
    __syncwarp();   // the scratch is rewritten by the next call
    if (!(owner && doit)) return;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    int16_t dout = inv;
    float cout = 0.0f;
    if constexpr (PYR) {
        int lo, hi;
        label_range(J, x, base, lo, hi);
        const int vc = hi >= lo ? hi - lo + 1 : 0;
        bool ok = vc >= 3 && minCost < kMax && alt < kMax;
        if (ok && J.uniq > 0 && alt * (100 - J.uniq) < minCost * 100) ok = false;
        const int realBest = base + bestD;
        const int physMax = imin(J.maxD, x);
        if ((bestD == 0 && base > J.minD) || (bestD == D - 1 && base + D - 1 < physMax)) ok = false;
        float cf = 0.0f;
        if (ok) {
            const float den = fmaxf((float)minCost, 1.0f);
            cf = fminf(fmaxf(((float)alt - (float)minCost) / den, 0.0f), 1.0f);
            if (cf < J.minConf) ok = false;
        }
        if (ok) {
            int d16 = realBest * 16;
            if (bestD > 0 && bestD + 1 < D && c0 < kMax && c1 < kMax && c2 < kMax) {
                const int den2 = imax(c0 + c2 - 2 * c1, 1);
                d16 += ((c0 - c2) * 16 + den2) / (den2 * 2);
            }
            dout = (int16_t)d16;
            cout = cf;
            const int x2 = x - realBest;
            if (x2 >= 0 && x2 < J.w)
                atomicMin(&J.keys[(size_t)y * J.w + x2], ((unsigned)minCost << 16) | (unsigned)(0xffff - x));
        }
    } else {
        bool unique = true;
        if (J.uniq > 0 && minCost < kMax / 2 && alt * (100 - J.uniq) < minCost * 100) unique = false;
        if (unique && minCost < kMax / 2) {
            int dint = bestD * 16;
            if (bestD > 0 && bestD < D - 1) {
                const int den2 = imax(c0 + c2 - 2 * c1, 1);
                dint = bestD * 16 + ((c0 - c2) * 16 + den2) / (den2 * 2);
            }
            dout = (int16_t)(dint + J.minD * 16);
            const int x2 = x - bestD - J.minD;
            if (x2 >= 0 && x2 < J.w)
                atomicMin(&J.keys[(size_t)y * J.w + x2], ((unsigned)minCost << 16) | (unsigned)(0xffff - x));
            const float den = fmaxf((float)minCost, 1.0f);
            cout = fminf(fmaxf(((float)alt - (float)minCost) / den, 0.0f), 1.0f);
        }
    }
    const size_t p = (size_t)y * J.w + x;
    J.disp_raw[p] = dout;
    J.conf_raw[p] = cout;
}

// Inputs of one pixel, loaded kPF steps ahead.
struct GPre {
    uint4 c;
    uint4 v;
    int base;
    int img;
};

template <bool PYR>
__device__ __forceinline__ void gprefetch(const LevelDesc& J, int y, int x, int k, int D, bool need_v, GPre& f)
{
    const size_t p = (size_t)y * J.w + x;
    const size_t o = p * D + 8 * k;
    f.c = __ldg(reinterpret_cast<const uint4*>(J.C + o));
    if (need_v) f.v = *reinterpret_cast<const uint4*>(J.V + o);   // may hold this kernel's own partials
    f.base = (PYR && J.refine) ? (int)__ldg(J.base + p) : J.minD;
    f.img = J.adaptive ? (int)__ldg(J.left + (size_t)y * J.lstep + x) : 0;
}

}  // namespace pk

// ---------------------------------------------------------------------------
// Top -> bottom: a warp holds 32/T adjacent columns, T threads each.
// ---------------------------------------------------------------------------
template <int T, bool PYR, int NJ>
__global__ void __launch_bounds__(pk::kWarps * 32) k_gtb(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<T>;
    constexpr int D = G::D;
    const LevelDesc& J = jobs.d[blockIdx.y];
    __shared__ int lut[256];
    __shared__ __align__(16) uint32_t cbuf[kWarps * 2 * G::BUFW];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * 2 * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lane / T, k = lane % T;
    int xlo = 0, xhi = J.w;
    if (!PYR) { xlo = imax(J.minD + D, 0); xhi = J.w + imin(J.minD, 0); }
    const int ncol = xhi - xlo;
    const int col0 = (blockIdx.x * kWarps + warp) * G::CPW;
    if (col0 >= ncol) return;   // the whole warp is past the image
    const int col = col0 + c;
    const bool col_ok = col < ncol;
    const int x = xlo + imin(col, ncol - 1), H = J.h;
    uint32_t* bufs = cbuf + warp * 2 * G::BUFW + G::off(c);
    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    int lo = 0, hi = D - 1;
    if (PYR && !J.refine) label_range(J, x, J.minD, lo, hi);
    GChain<T> s;
    gchain_init(s, J.minD);
    GPre ring[kPF] = {};
#pragma unroll
    for (int j = 0; j < kPF; ++j)
        if (j < H) gprefetch<PYR>(J, j, x, k, D, false, ring[j]);
    int img_prev = 0;
    for (int y0 = 0; y0 < H; y0 += kPF) {
#pragma unroll
        for (int j = 0; j < kPF; ++j) {
            const int y = y0 + j;
            if (y >= H) break;
            const GPre cur = ring[j];
            if (y + kPF < H) gprefetch<PYR>(J, y + kPF, x, k, D, false, ring[j]);
            const int p2 = J.adaptive ? lut[abs(cur.img - img_prev) & 255] : J.P2;
            img_prev = cur.img;
            uint32_t cc[4];
            to4(cur.c, cc);
            if (PYR && !J.refine) mask_labels<T>(cc, lo, hi, k);
            gstep<T, PYR>(s, cc, cur.base, p2, p12, bufs + (y & 1) * G::BUFW, k);
            if (col_ok)
                *reinterpret_cast<uint4*>(J.V + ((size_t)y * J.w + x) * D + 8 * k) = from4(s.L);
        }
    }
}

// ---------------------------------------------------------------------------
// Horizontal pass: a warp holds 16/T rows; per row an L->R group and an
// R->L group of T threads.
// ---------------------------------------------------------------------------
template <int T, bool PYR, int NJ>
__global__ void __launch_bounds__(pk::kWarps * 32) k_grow(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<T>;
    constexpr int D = G::D, DW = D / 2, RPW = G::CPW / 2, NB = kPF + 3;
    const LevelDesc& J = jobs.d[blockIdx.y];
    __shared__ int lut[256];
    __shared__ __align__(16) uint32_t cbuf[kWarps * 2 * G::BUFW];
    __shared__ __align__(16) uint32_t scrb[kWarps * 128];
    __shared__ __align__(16) uint32_t bandb[kWarps * RPW * NB * DW];
    __shared__ __align__(16) uint32_t midb[kWarps * RPW * DW];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * 2 * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lane / T, k = lane % T, r = c >> 1, dir = c & 1;
    const int row0 = (blockIdx.x * kWarps + warp) * RPW;
    if (row0 >= J.h) return;   // the whole warp is past the image
    const int y = row0 + r;
    const bool row_ok = y < J.h;
    const int yy = imin(y, J.h - 1);
    const int W = J.w;
    uint32_t* bufs = cbuf + warp * 2 * G::BUFW + G::off(c);
    uint32_t* band = bandb + (warp * RPW + r) * NB * DW;
    uint32_t* mid = midb + (warp * RPW + r) * DW;
    uint32_t* scr = scrb + warp * 128;

    // path extents (single-scale: kernel_AggregateLR/RL ranges)
    int minX1 = 0, maxX1 = W, lr_x0 = 0, lr_n, rl_n;
    if (PYR) {
        lr_n = J.paths >= 2 ? W : 0;
        rl_n = W;
    } else {
        minX1 = imax(J.minD + D, 0);
        maxX1 = W + imin(J.minD, 0);
        lr_x0 = minX1;
        lr_n = J.paths >= 2 ? imax(0, maxX1 - minX1) : 0;
        rl_n = imax(0, W - minX1);
    }
    const bool has_lr = lr_n > 0, has_tb = J.paths >= 3;
    const int n_mine = dir == 0 ? lr_n : rl_n;
    const int Tn = imax(lr_n, rl_n);
    const int C2 = W - 1 + lr_x0;                  // 2x at the meeting point
    const int band_lo = (C2 - kPF - 1 + 1) >> 1;   // first x with |2x - C2| <= kPF + 1
    auto in_band = [&](int x) { return abs(2 * x - C2) <= kPF + 1; };
    auto lr_covers = [&](int x) { return has_lr && x >= lr_x0 && x < lr_x0 + lr_n; };
    auto rl_covers = [&](int x) { return x >= W - rl_n; };
    auto wta_px = [&](int x) { return PYR || (x >= minX1 && x < maxX1 && x != W - 1); };
    auto xpos = [&](int t) {
        return dir == 0 ? lr_x0 + imin(t, imax(lr_n - 1, 0)) : W - 1 - imin(t, imax(rl_n - 1, 0));
    };
    // 0 nothing, 1 first at x, 2 second at x, 3 R->L alone, 4 R->L meets L->R at the same step
    auto role = [&](int t, int x) -> int {
        if (t >= n_mine) return 0;
        if (dir == 0) return rl_covers(x) ? ((W - 1 - x) < t ? 2 : 1) : 0;
        if (!has_lr) return 3;
        if (!lr_covers(x)) return 0;
        const int tl = x - lr_x0;
        return tl < t ? 2 : (tl == t ? 4 : 1);
    };
    auto need_v = [&](int ro, int x) { return (ro == 1 && has_tb) || (ro == 2 && !in_band(x)); };
    auto prefetch = [&](int t, GPre& f) {
        const int x = xpos(t);
        gprefetch<PYR>(J, yy, x, k, D, need_v(role(t, x), x), f);
    };

    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    GChain<T> s;
    gchain_init(s, J.minD);
    GPre ring[kPF] = {};
#pragma unroll
    for (int j = 0; j < kPF; ++j)
        if (j < n_mine) prefetch(j, ring[j]);
    int img_prev = 0;
    bool defer = false;
    int xm = 0, base_m = 0;
    for (int t0 = 0; t0 < Tn; t0 += kPF) {
#pragma unroll
        for (int j = 0; j < kPF; ++j) {
            const int t = t0 + j;
            if (t >= Tn) break;
            const int x = xpos(t);
            const GPre cur = ring[j];
            if (t + kPF < n_mine) prefetch(t + kPF, ring[j]);
            const int p2 = J.adaptive ? lut[abs(cur.img - img_prev) & 255] : J.P2;
            img_prev = cur.img;
            uint32_t cc[4];
            to4(cur.c, cc);
            if (PYR && !J.refine) {
                int lo, hi;
                label_range(J, x, J.minD, lo, hi);
                mask_labels<T>(cc, lo, hi, k);
            }
            gstep<T, PYR>(s, cc, cur.base, p2, p12, bufs + (t & 1) * G::BUFW, k);
            const int ro = role(t, x);
            uint32_t vin[4], tot[4] = {kMax2, kMax2, kMax2, kMax2};
            to4(cur.v, vin);
            uint4* slot = reinterpret_cast<uint4*>(band + (x - band_lo) * DW) + k;
            uint4* vout = reinterpret_cast<uint4*>(J.V + ((size_t)yy * W + x) * D + 8 * k);
            if (ro == 1) {
                uint32_t part[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) part[i] = has_tb ? gcombine<PYR>(s.L[i], vin[i]) : s.L[i];
                if (in_band(x)) *slot = from4(part);
                else if (row_ok) *vout = from4(part);
            } else if (ro == 4) {
                reinterpret_cast<uint4*>(mid)[k] = from4(s.L);
                defer = true;
                xm = x;
                base_m = cur.base;
            } else if (ro == 2) {
                uint32_t part[4];
                if (in_band(x)) to4(*slot, part);
                else to4(cur.v, part);
#pragma unroll
                for (int i = 0; i < 4; ++i) tot[i] = gcombine<PYR>(part[i], s.L[i]);
                if (J.debug_acc && row_ok) *vout = from4(tot);
            } else if (ro == 3) {
#pragma unroll
                for (int i = 0; i < 4; ++i) tot[i] = s.L[i];
                if (J.debug_acc && row_ok) *vout = from4(tot);
            }
            const bool wta = (ro == 2 || ro == 3) && wta_px(x);
            if (__any_sync(0xffffffffu, wta)) gwta<T, PYR>(J, wta && row_ok, yy, x, tot, cur.base, scr, lane, k);
        }
    }
    __syncwarp();
    {
        // the pixel both paths reach at the same step: R->L finishes it
        uint32_t tot[4] = {kMax2, kMax2, kMax2, kMax2};
        bool wta = false;
        if (defer) {
            uint32_t part[4], lm[4];
            to4(reinterpret_cast<const uint4*>(band + (xm - band_lo) * DW)[k], part);
            to4(reinterpret_cast<const uint4*>(mid)[k], lm);
#pragma unroll
            for (int i = 0; i < 4; ++i) tot[i] = gcombine<PYR>(part[i], lm[i]);
            if (J.debug_acc && row_ok)
                *reinterpret_cast<uint4*>(J.V + ((size_t)yy * W + xm) * D + 8 * k) = from4(tot);
            wta = wta_px(xm);
        }
        if (__any_sync(0xffffffffu, wta)) gwta<T, PYR>(J, wta && row_ok, yy, xm, tot, base_m, scr, lane, k);
    }
    // single-scale: pixels no path finishes stay invalid
    if (!PYR && row_ok) {
        const int16_t inv = (int16_t)((J.minD - 1) * 16);
        for (int x = dir * T + k; x < W; x += 2 * T) {
            if (wta_px(x)) continue;
            J.disp_raw[(size_t)y * W + x] = inv;
            J.conf_raw[(size_t)y * W + x] = 0.0f;
        }
    }
}

template <int T, bool PYR, int NJ>
cudaError_t launch_paths_packed(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    using G = pk::Grp<T>;
    cudaError_t err;
    bool any_tb = false;
    for (int i = 0; i < jobs.n; ++i) any_tb = any_tb || jobs.d[i].paths >= 3;
    if (any_tb) {
        Jobs<NJ> tbj = jobs;
        int n = 0;
        for (int i = 0; i < jobs.n; ++i)
            if (jobs.d[i].paths >= 3) tbj.d[n++] = jobs.d[i];
        tbj.n = n;
        const int cols = pk::kWarps * G::CPW;
        dim3 g((e.max_w + cols - 1) / cols, n);
        prof_begin(st);
        k_gtb<T, PYR, NJ><<<g, pk::kWarps * 32, 0, st>>>(tbj);
        count_launch();
        prof_end(PK_PATH_TB, jobs_vox(tbj) * 4 + jobs_px(tbj) * (tbj.d[0].refine ? 2 : 0), st);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    const int rows = pk::kWarps * G::CPW / 2;
    dim3 g((e.max_h + rows - 1) / rows, jobs.n);
    prof_begin(st);
    k_grow<T, PYR, NJ><<<g, pk::kWarps * 32, 0, st>>>(jobs);
    count_launch();
    if (prof_enabled()) {
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double px = (double)d.w * d.h;
            by += px * d.D * (2 + (d.paths >= 3 ? 2 : 0)) + px * (6 + (d.refine ? 2 : 0));
        }
        prof_end(PK_PATH_ROW, by, st);
    }
    return cudaGetLastError();
}

}  // namespace pg
