// k_paths.cuh -- SGM path aggregation and winner-take-all.
//
// Reference semantics (reference file:line):
//   single-scale  kernel_SGM_PathLR / PathTB / PathRL_WTA, src/sgm_kernels.cu:520-819
//   pyramid       kernel_SGM_PathLRPyramid / TBPyramid / RLPyramidWTA,
//                 src/sgm_kernels.cu:1191-1478
//   LR checks     kernel_PseudoLRCheck / kernel_StrictPyramidLRCheck,
//                 src/sgm_kernels.cu:825-889
//
// Design.  A path chain (one image row for L->R / R->L, one column for
// T->B) is owned by a group of G lanes (16 or 32), each holding K labels
// (blocked layout: lane l owns labels l*K .. l*K+K-1).  Per pixel the
// recurrence needs the previous pixel's costs at the mapped labels
// same = d + base - prevBase and same +- 1 (warp shuffles for K == 1,
// a warp-private shared buffer otherwise) and the minimum over all labels
// (a group reduction).  Labels D..G*K-1 are padding and stay invalid.
//
// The T->B kernel writes its path costs to the aggregation volume V.  The
// row kernel then runs L->R and R->L of the same row in the same lanes,
// interleaved (two independent dependency chains per warp).  The path that
// reaches a pixel first leaves its partial sum (with the T->B cost folded
// in) in V; the one that arrives second adds its own cost and finishes the
// pixel: packed-key argmin, second minimum, uniqueness, confidence,
// sub-pixel and the right-image disparity (disp2).  The reference's
// clamped sums are order independent -- every term is non-negative and is
// clamped at one cap (SHRT_MAX single-scale; SHRT_MAX-1 with a SHRT_MAX
// sentinel in the pyramid) -- so the totals equal the reference's
// L->R, T->B, R->L accumulation exactly.
//
// disp2 in the reference is written right to left and keeps the first
// strictly smaller cost, i.e. for every target column the minimum cost
// with ties going to the largest source column.  Here every candidate does
// atomicMin on (cost << 16 | (0xFFFF - x)) in a per-row shared array, which
// selects the same winner independent of the visiting order; the winner's
// disparity is x - x2.  After both passes the row's LR check reads that
// array directly.
#pragma once

#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {

constexpr unsigned kFull = 0xffffffffu;
constexpr unsigned kNoKey = 0xffffffffu;

template <int G>
__device__ __forceinline__ int group_min(int v)
{
    if constexpr (G == 32) {
        return __reduce_min_sync(kFull, v);
    } else {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) v = imin(v, __shfl_xor_sync(kFull, v, o, G));
        return v;
    }
}

template <int G>
__device__ __forceinline__ unsigned group_min_u(unsigned v)
{
    if constexpr (G == 32) {
        return __reduce_min_sync(kFull, v);
    } else {
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            const unsigned w = __shfl_xor_sync(kFull, v, o, G);
            v = w < v ? w : v;
        }
        return v;
    }
}

// K consecutive int16 values starting at a K*2-byte aligned address.
template <int K>
__device__ __forceinline__ void load_k(const int16_t* src, int (&v)[K])
{
    if constexpr (K == 1) {
        v[0] = src[0];
    } else if constexpr (K == 2) {
        const uint32_t u = *reinterpret_cast<const uint32_t*>(src);
        v[0] = (int16_t)(u & 0xffff);
        v[1] = (int16_t)(u >> 16);
    } else if constexpr (K == 4) {
        const uint2 u = *reinterpret_cast<const uint2*>(src);
        v[0] = (int16_t)(u.x & 0xffff); v[1] = (int16_t)(u.x >> 16);
        v[2] = (int16_t)(u.y & 0xffff); v[3] = (int16_t)(u.y >> 16);
    } else {
#pragma unroll
        for (int i = 0; i < K / 8; ++i) {
            const uint4 u = reinterpret_cast<const uint4*>(src)[i];
            const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v[8 * i + 2 * j] = (int16_t)(w[j] & 0xffff);
                v[8 * i + 2 * j + 1] = (int16_t)(w[j] >> 16);
            }
        }
    }
}

template <int K>
__device__ __forceinline__ void store_k(int16_t* dst, const int (&v)[K])
{
    if constexpr (K == 1) {
        dst[0] = (int16_t)v[0];
    } else if constexpr (K == 2) {
        *reinterpret_cast<uint32_t*>(dst) = (uint32_t)(uint16_t)v[0] | ((uint32_t)(uint16_t)v[1] << 16);
    } else if constexpr (K == 4) {
        uint2 u;
        u.x = (uint32_t)(uint16_t)v[0] | ((uint32_t)(uint16_t)v[1] << 16);
        u.y = (uint32_t)(uint16_t)v[2] | ((uint32_t)(uint16_t)v[3] << 16);
        *reinterpret_cast<uint2*>(dst) = u;
    } else {
#pragma unroll
        for (int i = 0; i < K / 8; ++i) {
            uint32_t w[4];
#pragma unroll
            for (int j = 0; j < 4; ++j)
                w[j] = (uint32_t)(uint16_t)v[8 * i + 2 * j] | ((uint32_t)(uint16_t)v[8 * i + 2 * j + 1] << 16);
            reinterpret_cast<uint4*>(dst)[i] = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// Volume element access for the labels of lane gl; labels >= D read as kMax.
template <int K>
__device__ __forceinline__ void load_labels(const int16_t* pix, int D, int gl, int (&v)[K])
{
    const int d0 = gl * K;
    if (d0 + K <= D) {
        load_k<K>(pix + d0, v);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] = (d0 + k < D) ? (int)pix[d0 + k] : kMax;
    }
}

template <int K>
__device__ __forceinline__ void store_labels(int16_t* pix, int D, int gl, const int (&v)[K])
{
    const int d0 = gl * K;
    if (d0 + K <= D) {
        store_k<K>(pix + d0, v);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (d0 + k < D) pix[d0 + k] = (int16_t)v[k];
    }
}

template <int K>
struct Chain {
    int L[K];
    int minPrev;
    int prevBase;
    bool active;  // the previous pixel had at least one finite path cost
    int par;      // exchange-buffer parity (K > 1)
};

template <int K>
__device__ __forceinline__ void chain_init(Chain<K>& s, int minD)
{
#pragma unroll
    for (int k = 0; k < K; ++k) s.L[k] = kMax;
    s.minPrev = kMax;
    s.prevBase = minD;
    s.active = false;
    s.par = 0;
}

// Inputs of one chain step at one pixel.
template <int K>
struct StepIn {
    int c[K];     // matching cost (kMax for an invalid label in pyramid mode)
    bool lv[K];   // label valid (pyramid)
    int vc;       // number of geometry-valid labels (pyramid)
    int base;     // real disparity of local label 0
    int p2;       // effective P2 towards the previous pixel
};

template <int K, bool PYR>
__device__ __forceinline__ void load_step(const LevelDesc& J, int y, int x, int gl, StepIn<K>& in)
{
    const size_t p = (size_t)y * J.w + x;
    load_labels<K>(J.C + p * J.D, J.D, gl, in.c);
    if constexpr (PYR) {
        in.base = J.refine ? (int)J.base[p] : J.minD;
        int lo, hi;
        label_range(J, x, in.base, lo, hi);
        in.vc = hi >= lo ? hi - lo + 1 : 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int d = gl * K + k;
            in.lv[k] = d >= lo && d <= hi && in.c[k] < kMax;
            if (!in.lv[k]) in.c[k] = kMax;
        }
    } else {
        in.base = J.minD;
        in.vc = J.D;
#pragma unroll
        for (int k = 0; k < K; ++k) in.lv[k] = gl * K + k < J.D;
    }
}

// One step of the path recurrence (src/sgm_kernels.cu:560-565 single-scale,
// 1230-1252 pyramid).  All lanes of the warp must call it together.
// xb: this chain's exchange buffer, 2 x (G*K) int16 (K > 1 only).
template <int G, int K, bool PYR>
__device__ __forceinline__ void chain_step(Chain<K>& s, const StepIn<K>& in, int P1, int D, int gl,
                                           int16_t* xb, int (&Lc)[K])
{
    const int delta = PYR ? in.base - s.prevBase : 0;
    int n0[K], nm[K], np[K];
    if constexpr (K == 1) {
        const int si = gl + delta;
        const int v0 = __shfl_sync(kFull, s.L[0], iclamp(si, 0, G - 1), G);
        const int vm = __shfl_sync(kFull, s.L[0], iclamp(si - 1, 0, G - 1), G);
        const int vp = __shfl_sync(kFull, s.L[0], iclamp(si + 1, 0, G - 1), G);
        n0[0] = (si >= 0 && si < D) ? v0 : kMax;
        nm[0] = (si - 1 >= 0 && si - 1 < D) ? imin(kMax, vm + P1) : kMax;
        np[0] = (si + 1 >= 0 && si + 1 < D) ? imin(kMax, vp + P1) : kMax;
    } else {
        int16_t* buf = xb + s.par * (G * K);
#pragma unroll
        for (int k = 0; k < K; ++k) buf[gl * K + k] = (int16_t)s.L[k];
        __syncwarp();
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int si = gl * K + k + delta;
            n0[k] = (si >= 0 && si < D) ? (int)buf[si] : kMax;
            nm[k] = (si - 1 >= 0 && si - 1 < D) ? imin(kMax, (int)buf[si - 1] + P1) : kMax;
            np[k] = (si + 1 >= 0 && si + 1 < D) ? imin(kMax, (int)buf[si + 1] + P1) : kMax;
        }
        s.par ^= 1;
    }
    const int lj = imin(kMax, s.minPrev + in.p2);
    int m = kMax;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int best = imin(imin(n0[k], nm[k]), imin(np[k], lj));
        int v;
        if constexpr (PYR) {
            v = !s.active ? in.c[k]
                          : (!in.lv[k] ? kMax : (best < kMax ? sat16(in.c[k] + best - s.minPrev) : kMax));
            if (in.vc == 0) v = kMax;
        } else {
            v = !s.active ? in.c[k] : sat16(in.c[k] + best - s.minPrev);
            if (!in.lv[k]) v = kMax;  // padding labels
        }
        Lc[k] = v;
        m = imin(m, v);
    }
    const int minCur = group_min<G>(m);
#pragma unroll
    for (int k = 0; k < K; ++k) s.L[k] = Lc[k];
    s.minPrev = minCur;
    s.prevBase = in.base;
    s.active = PYR ? (in.vc > 0 && minCur < kMax) : true;
}

// Partial sum left by the first horizontal path to reach a pixel.
template <int K, bool PYR>
__device__ __forceinline__ void combine_first(const int (&L)[K], const int (&tb)[K], bool has_tb, int (&out)[K])
{
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int t = has_tb ? tb[k] : 0;
        if constexpr (PYR) out[k] = (L[k] < kMax && t < kMax) ? imin(kMax - 1, L[k] + t) : kMax;
        else out[k] = imin(kMax, L[k] + t);
    }
}

// Total when the second horizontal path reaches the pixel.
template <int K, bool PYR>
__device__ __forceinline__ void combine_second(const int (&part)[K], const int (&L)[K], int (&tot)[K])
{
#pragma unroll
    for (int k = 0; k < K; ++k) {
        if constexpr (PYR) tot[k] = (part[k] < kMax && L[k] < kMax) ? imin(kMax - 1, part[k] + L[k]) : kMax;
        else tot[k] = imin(kMax, part[k] + L[k]);
    }
}

__device__ __forceinline__ unsigned disp2_key(int cost, int x)
{
    return ((unsigned)cost << 16) | (unsigned)(0xffff - x);
}

// Winner-take-all of one pixel from the final aggregated costs.
// Single-scale: src/sgm_kernels.cu:744-808.  Pyramid: 1413-1471.
template <int G, int K, bool PYR>
__device__ __forceinline__ void wta(const LevelDesc& J, int y, int x, const int (&tot)[K], const StepIn<K>& in,
                                    int gl, unsigned* keys, bool active)
{
    const int D = J.D;
    unsigned km = kNoKey;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int d = gl * K + k;
        const unsigned key = ((unsigned)(uint16_t)tot[k] << 16) | (unsigned)d;
        if (d < D && key < km) km = key;
    }
    const unsigned best = group_min_u<G>(km);
    const int minCost = (int)(best >> 16);
    const int bestD = (int)(best & 0xffffu);
    int am = kMax;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int d = gl * K + k;
        const int dd = d - bestD;
        if (d < D && (dd > 1 || dd < -1) && (!PYR || in.lv[k])) am = imin(am, tot[k]);
    }
    const int alt = group_min<G>(am);
    int nb[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int b = bestD - 1 + j;
        int v = 0;
#pragma unroll
        for (int k = 0; k < K; ++k)
            if (gl * K + k == b) v = tot[k];
        nb[j] = __shfl_sync(kFull, v, iclamp(b, 0, D - 1) / K, G);
    }
    if (gl != 0 || !active) return;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    const size_t p = (size_t)y * J.w + x;
    int16_t dout = inv;
    float cout = 0.0f;
    if constexpr (PYR) {
        bool ok = in.vc >= 3 && minCost < kMax && alt < kMax;
        if (ok && J.uniq > 0 && alt * (100 - J.uniq) < minCost * 100) ok = false;
        const int realBest = in.base + bestD;
        const int physMax = imin(J.maxD, x);
        if ((bestD == 0 && in.base > J.minD) || (bestD == D - 1 && in.base + D - 1 < physMax)) ok = false;
        float c = 0.0f;
        if (ok) {
            const float den = fmaxf((float)minCost, 1.0f);
            c = fminf(fmaxf(((float)alt - (float)minCost) / den, 0.0f), 1.0f);
            if (c < J.minConf) ok = false;
        }
        if (ok) {
            int d16 = realBest * 16;
            if (bestD > 0 && bestD + 1 < D && nb[0] < kMax && nb[1] < kMax && nb[2] < kMax) {
                const int den2 = imax(nb[0] + nb[2] - 2 * nb[1], 1);
                d16 += ((nb[0] - nb[2]) * 16 + den2) / (den2 * 2);
            }
            dout = (int16_t)d16;
            cout = c;
            const int x2 = x - realBest;
            if (x2 >= 0 && x2 < J.w) atomicMin(&keys[x2], disp2_key(minCost, x));
        }
    } else {
        bool unique = true;
        if (J.uniq > 0 && minCost < kMax / 2 && alt * (100 - J.uniq) < minCost * 100) unique = false;
        if (unique && minCost < kMax / 2) {
            int dint = bestD * 16;
            if (bestD > 0 && bestD < D - 1) {
                const int den2 = imax(nb[0] + nb[2] - 2 * nb[1], 1);
                dint = bestD * 16 + ((nb[0] - nb[2]) * 16 + den2) / (den2 * 2);
            }
            dout = (int16_t)(dint + J.minD * 16);
            const int x2 = x - bestD - J.minD;
            if (x2 >= 0 && x2 < J.w) atomicMin(&keys[x2], disp2_key(minCost, x));
            const float den = fmaxf((float)minCost, 1.0f);
            cout = fminf(fmaxf(((float)alt - (float)minCost) / den, 0.0f), 1.0f);
        }
    }
    J.disp_raw[p] = dout;
    J.conf_raw[p] = cout;
}

// ---------------------------------------------------------------------------
// Top -> bottom path.  Block: 4 warps; each warp owns 32/G columns.
// ---------------------------------------------------------------------------
constexpr int kTbWarps = 4;

template <int G, int K, bool PYR, int NJ>
__global__ void __launch_bounds__(kTbWarps * 32) k_path_tb(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.y];
    constexpr int CPW = 32 / G;
    extern __shared__ __align__(16) unsigned char sm[];
    int* lut = reinterpret_cast<int*>(sm);
    if (J.adaptive)
        for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.p2lut[i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, gl = lane % G, grp = lane / G;
    int xlo = 0, xhi = J.w;
    if (!PYR) { xlo = imax(J.minD + J.D, 0); xhi = J.w + imin(J.minD, 0); }
    const int ncols = xhi - xlo;
    const int c0 = (blockIdx.x * kTbWarps + warp) * CPW;
    if (c0 >= ncols) return;
    const bool active = c0 + grp < ncols;
    const int x = xlo + (active ? c0 + grp : ncols - 1);
    int16_t* xb = reinterpret_cast<int16_t*>(sm + 1024) + (warp * CPW + grp) * (2 * G * K);
    Chain<K> s;
    chain_init(s, J.minD);
    for (int y = 0; y < J.h; ++y) {
        StepIn<K> in;
        load_step<K, PYR>(J, y, x, gl, in);
        in.p2 = J.P2;
        if (J.adaptive && s.active) {
            const int a = J.left[(size_t)y * J.lstep + x], b = J.left[(size_t)(y - 1) * J.lstep + x];
            in.p2 = lut[a > b ? a - b : b - a];
        }
        int L[K];
        chain_step<G, K, PYR>(s, in, J.P1, J.D, gl, xb, L);
        if (active) store_labels<K>(J.V + ((size_t)y * J.w + x) * J.D, J.D, gl, L);
    }
}

// ---------------------------------------------------------------------------
// Row kernel: L->R and R->L of one row, WTA, disp2, LR check.  One warp per
// block; each warp owns 32/G rows.
// ---------------------------------------------------------------------------
template <int G, int K, bool PYR, int NJ>
__global__ void __launch_bounds__(32) k_path_row(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.y];
    constexpr int RPW = 32 / G;
    const int W = J.w, H = J.h, D = J.D;
    const int y0 = blockIdx.x * RPW;
    if (y0 >= H) return;
    const int lane = threadIdx.x, gl = lane % G, grp = lane / G;
    const bool active = y0 + grp < H;
    const int y = active ? y0 + grp : H - 1;

    extern __shared__ __align__(16) unsigned char sm[];
    int* lut = reinterpret_cast<int*>(sm);
    unsigned* keys = reinterpret_cast<unsigned*>(sm + 1024) + grp * W;
    int16_t* xb = reinterpret_cast<int16_t*>(sm + 1024 + (size_t)RPW * W * 4) + grp * (4 * G * K);
    if (J.adaptive)
        for (int i = lane; i < 256; i += 32) lut[i] = J.p2lut[i];
    for (int x = gl; x < W; x += G) keys[x] = kNoKey;
    __syncwarp();

    const uint8_t* img = J.left + (size_t)y * J.lstep;
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
    const bool has_tb = J.paths >= 3;
    Chain<K> lr, rl;
    chain_init(lr, J.minD);
    chain_init(rl, J.minD);
    const int T = imax(lr_n, rl_n);
    for (int t = 0; t < T; ++t) {
        if (t < lr_n) {
            const int x = lr_x0 + t;
            StepIn<K> in;
            load_step<K, PYR>(J, y, x, gl, in);
            in.p2 = J.P2;
            if (J.adaptive && lr.active) {
                const int a = img[x], b = img[x - 1];
                in.p2 = lut[a > b ? a - b : b - a];
            }
            int L[K];
            chain_step<G, K, PYR>(lr, in, J.P1, D, gl, xb, L);
            int16_t* vp = J.V + ((size_t)y * W + x) * D;
            const bool rl_cov = x >= W - rl_n;
            if (rl_cov && (W - 1 - x) < t) {
                int part[K], tot[K];
                load_labels<K>(vp, D, gl, part);
                combine_second<K, PYR>(part, L, tot);
                if (J.debug_acc && active) store_labels<K>(vp, D, gl, tot);
                if (PYR || x != W - 1) wta<G, K, PYR>(J, y, x, tot, in, gl, keys, active);
            } else if (rl_cov) {
                int tb[K], part[K];
                if (has_tb) load_labels<K>(vp, D, gl, tb);
                combine_first<K, PYR>(L, tb, has_tb, part);
                if (active) store_labels<K>(vp, D, gl, part);
            }
        }
        if (t < rl_n) {
            const int x = W - 1 - t;
            StepIn<K> in;
            load_step<K, PYR>(J, y, x, gl, in);
            in.p2 = J.P2;
            if (J.adaptive && rl.active) {
                const int a = img[x], b = img[x + 1];
                in.p2 = lut[a > b ? a - b : b - a];
            }
            int L[K];
            chain_step<G, K, PYR>(rl, in, J.P1, D, gl, xb + 2 * G * K, L);
            int16_t* vp = J.V + ((size_t)y * W + x) * D;
            const bool wta_px = PYR || (x >= minX1 && x < maxX1 && x != W - 1);
            const bool lr_cov = lr_n > 0 && x >= lr_x0 && x < lr_x0 + lr_n;
            if (lr_n == 0) {
                // R->L is the only horizontal path (and there is no T->B)
                if (J.debug_acc && active) store_labels<K>(vp, D, gl, L);
                if (wta_px) wta<G, K, PYR>(J, y, x, L, in, gl, keys, active);
            } else if (lr_cov && (x - lr_x0) <= t) {
                int part[K], tot[K];
                load_labels<K>(vp, D, gl, part);
                combine_second<K, PYR>(part, L, tot);
                if (J.debug_acc && active) store_labels<K>(vp, D, gl, tot);
                if (wta_px) wta<G, K, PYR>(J, y, x, tot, in, gl, keys, active);
            } else if (lr_cov) {
                int tb[K], part[K];
                if (has_tb) load_labels<K>(vp, D, gl, tb);
                combine_first<K, PYR>(L, tb, has_tb, part);
                if (active) store_labels<K>(vp, D, gl, part);
            }
        }
    }
    __syncwarp();

    // LR check over the finished row and the final per-pixel write.
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    const bool check = (J.post & POST_LRCHECK) != 0;
    for (int x = gl; x < W; x += G) {
        const size_t p = (size_t)y * W + x;
        const bool wp = PYR || (x >= minX1 && x < maxX1 && x != W - 1);
        int d16 = inv;
        float cf = 0.0f;
        if (wp) { d16 = J.disp_raw[p]; cf = J.conf_raw[p]; }
        if (check && d16 != inv) {
            const int d0 = d16 >> 4, d1 = (d16 + 15) >> 4;
            const int r0 = x - d0, r1 = x - d1;
            auto disp2 = [&](int rx) -> int {
                const unsigned k = keys[rx];
                return k == kNoKey ? (int)inv : (int)(0xffffu - (k & 0xffffu)) - rx;
            };
            if (PYR) {
                bool ok = false;
                if (r0 >= 0 && r0 < W) { const int v = disp2(r0); if (v >= J.minD && abs(v - d0) <= J.maxdiff) ok = true; }
                if (r1 >= 0 && r1 < W) { const int v = disp2(r1); if (v >= J.minD && abs(v - d1) <= J.maxdiff) ok = true; }
                if (!ok) { d16 = inv; cf = 0.0f; }
            } else {
                bool bad0 = false, bad1 = false;
                if (r0 >= 0 && r0 < W) { const int v = disp2(r0); bad0 = v >= J.minD && abs(v - d0) > J.maxdiff; }
                if (r1 >= 0 && r1 < W) { const int v = disp2(r1); bad1 = v >= J.minD && abs(v - d1) > J.maxdiff; }
                if (bad0 && bad1) { d16 = inv; cf = 0.0f; }
            }
        }
        if (active) { J.disp_raw[p] = (int16_t)d16; J.conf_raw[p] = cf; }
    }
}

template <int G, int K, bool PYR, int NJ>
cudaError_t launch_paths_shape(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    cudaError_t err;
    bool any_tb = false;
    for (int i = 0; i < jobs.n; ++i) any_tb = any_tb || jobs.d[i].paths >= 3;
    if (any_tb) {
        const size_t smem = 1024 + (K > 1 ? (size_t)kTbWarps * 32 / G * 2 * G * K * 2 : 0);
        const int cols_per_block = kTbWarps * (32 / G);
        dim3 g((e.max_w + cols_per_block - 1) / cols_per_block, jobs.n);
        // jobs without T->B return at once: their columns count is taken as zero below
        Jobs<NJ> tbj = jobs;
        int n = 0;
        for (int i = 0; i < jobs.n; ++i)
            if (jobs.d[i].paths >= 3) tbj.d[n++] = jobs.d[i];
        tbj.n = n;
        g.y = n;
        prof_begin(st);
        k_path_tb<G, K, PYR, NJ><<<g, kTbWarps * 32, smem, st>>>(tbj);
        count_launch();
        // read C, write V (int16 per voxel); label base per pixel on refine levels
        prof_end(PK_PATH_TB, jobs_vox(tbj) * 4 + jobs_px(tbj) * (tbj.d[0].refine ? 2 : 0), st);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    constexpr int RPW = 32 / G;
    const size_t smem = 1024 + (size_t)RPW * e.max_w * 4 + (K > 1 ? (size_t)RPW * 4 * G * K * 2 : 0);
    if (smem > 48 * 1024) {
        err = cudaFuncSetAttribute(k_path_row<G, K, PYR, NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
    }
    dim3 g((e.max_h + RPW - 1) / RPW, jobs.n);
    prof_begin(st);
    k_path_row<G, K, PYR, NJ><<<g, 32, smem, st>>>(jobs);
    count_launch();
    if (prof_enabled()) {
        // read C and the T->B volume, write disparity and confidence (and read the label base)
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

template <bool PYR, int NJ>
cudaError_t launch_paths_mode(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    const PathShape s = path_shape(jobs.d[0].D);
    switch (s.G * 100 + s.K) {
    case 1601: return launch_paths_shape<16, 1, PYR, NJ>(jobs, e, st);
    case 3201: return launch_paths_shape<32, 1, PYR, NJ>(jobs, e, st);
    case 3202: return launch_paths_shape<32, 2, PYR, NJ>(jobs, e, st);
    case 3204: return launch_paths_shape<32, 4, PYR, NJ>(jobs, e, st);
    case 3208: return launch_paths_shape<32, 8, PYR, NJ>(jobs, e, st);
    case 3216: return launch_paths_shape<32, 16, PYR, NJ>(jobs, e, st);
    case 3232: return launch_paths_shape<32, 32, PYR, NJ>(jobs, e, st);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace pg
