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

#include <algorithm>
#include <climits>

#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"
#include "k_paths_packed.cuh"
#include "k_fused.cuh"

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
    bool lv[K];   // label valid (pyramid); label < D (single-scale)
    int vc;       // number of geometry-valid labels (pyramid)
    int base;     // real disparity of local label 0
    int p2;       // effective P2 towards the previous pixel
};

// Global inputs of one chain step are loaded pf_depth<K>() steps ahead of
// their use so that no load latency sits on the serial recurrence (deep for
// few labels per lane, shallower where the ring would spill registers).
template <int K>
__host__ __device__ constexpr int pf_depth()
{
    return K <= 2 ? 8 : (K <= 8 ? 4 : 2);
}

template <int K>
struct Pre {
    int c[K];     // cost volume C
    int v[K];     // aggregation volume V (T->B cost or a first-arrival partial), when needed
    int base;     // label base (refine levels)
    int img;      // left intensity (adaptive P2)
};

template <int K>
__device__ __forceinline__ void load_k_ro(const int16_t* src, int (&v)[K])
{
    if constexpr (K == 1) {
        v[0] = __ldg(src);
    } else if constexpr (K == 2) {
        const uint32_t u = __ldg(reinterpret_cast<const unsigned int*>(src));
        v[0] = (int16_t)(u & 0xffff);
        v[1] = (int16_t)(u >> 16);
    } else if constexpr (K == 4) {
        const uint2 u = __ldg(reinterpret_cast<const uint2*>(src));
        v[0] = (int16_t)(u.x & 0xffff); v[1] = (int16_t)(u.x >> 16);
        v[2] = (int16_t)(u.y & 0xffff); v[3] = (int16_t)(u.y >> 16);
    } else {
#pragma unroll
        for (int i = 0; i < K / 8; ++i) {
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(src) + i);
            const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                v[8 * i + 2 * j] = (int16_t)(w[j] & 0xffff);
                v[8 * i + 2 * j + 1] = (int16_t)(w[j] >> 16);
            }
        }
    }
}

template <int K, bool PYR>
__device__ __forceinline__ void prefetch(const LevelDesc& J, int y, int x, int gl, bool need_v, Pre<K>& f)
{
    const size_t p = (size_t)y * J.w + x;
    const int16_t* cp = J.C + p * J.D;
    const int d0 = gl * K;
    if (d0 + K <= J.D) {
        load_k_ro<K>(cp + d0, f.c);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k) f.c[k] = (d0 + k < J.D) ? (int)__ldg(cp + d0 + k) : kMax;
    }
    if (need_v) load_labels<K>(J.V + p * J.D, J.D, gl, f.v);
    f.base = (PYR && J.refine) ? (int)__ldg(J.base + p) : J.minD;
    f.img = J.adaptive ? (int)__ldg(J.left + (size_t)y * J.lstep + x) : 0;
}

// Label validity of pixel x from its prefetched inputs.
template <int K, bool PYR>
__device__ __forceinline__ void make_step(const LevelDesc& J, int x, int gl, const Pre<K>& f, StepIn<K>& in)
{
    in.base = f.base;
    if constexpr (PYR) {
        int lo, hi;
        label_range(J, x, f.base, lo, hi);
        in.vc = hi >= lo ? hi - lo + 1 : 0;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int d = gl * K + k;
            in.lv[k] = d >= lo && d <= hi && f.c[k] < kMax;
            in.c[k] = in.lv[k] ? f.c[k] : kMax;
        }
    } else {
        in.vc = J.D;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            in.lv[k] = gl * K + k < J.D;
            in.c[k] = f.c[k];
        }
    }
}

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

// ---------------------------------------------------------------------------
// Top -> bottom path.  Block: 4 warps; each warp owns 32/G columns.  The
// cost, label base and intensity of row y + kPF are loaded while row y is
// aggregated.
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
    const int H = J.h;
    int16_t* xb = reinterpret_cast<int16_t*>(sm + 1024) + (warp * CPW + grp) * (2 * G * K);
    constexpr int kPF = pf_depth<K>();
    Chain<K> s;
    chain_init(s, J.minD);
    Pre<K> ring[kPF];
#pragma unroll
    for (int j = 0; j < kPF; ++j)
        if (j < H) prefetch<K, PYR>(J, j, x, gl, false, ring[j]);
    int img_prev = 0;
    for (int y0 = 0; y0 < H; y0 += kPF) {
#pragma unroll
        for (int j = 0; j < kPF; ++j) {
            const int y = y0 + j;
            if (y < H) {
                StepIn<K> in;
                make_step<K, PYR>(J, x, gl, ring[j], in);
                const int img = ring[j].img;
                in.p2 = (J.adaptive && s.active) ? lut[abs(img - img_prev) & 255] : J.P2;
                img_prev = img;
                if (y + kPF < H) prefetch<K, PYR>(J, y + kPF, x, gl, false, ring[j]);
                int L[K];
                chain_step<G, K, PYR>(s, in, J.P1, J.D, gl, xb, L);
                if (active && PG_IN(((size_t)y * J.w + x) * J.D, J.D, (size_t)J.w * H * J.D, 12))
                    store_labels<K>(J.V + ((size_t)y * J.w + x) * J.D, J.D, gl, L);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Winner-take-all of one pixel from its final aggregated costs, one lane per
// pixel (deferred: the row kernel stashes each finished pixel's costs and
// every G steps each lane finishes one of them).
// Single-scale: src/sgm_kernels.cu:744-808.  Pyramid: 1413-1471.
// tot: the pixel's D costs (16-byte aligned, D a multiple of 16).
// ---------------------------------------------------------------------------
template <bool PYR>
__device__ __forceinline__ void finish_pixel(const LevelDesc& J, int y, int x, const int16_t* tot, int base, int vc,
                                             unsigned* keys)
{
    const int D = J.D;
    unsigned best = kNoKey;
    for (int c = 0; c < D; c += 8) {
        const uint4 q = *reinterpret_cast<const uint4*>(tot + c);
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const unsigned k0 = ((w[i] & 0xffffu) << 16) | (unsigned)(c + 2 * i);
            const unsigned k1 = (w[i] & 0xffff0000u) | (unsigned)(c + 2 * i + 1);
            best = k0 < best ? k0 : best;
            best = k1 < best ? k1 : best;
        }
    }
    const int minCost = (int)(best >> 16);
    const int bestD = (int)(best & 0xffffu);
    int alt = kMax;
    for (int c = 0; c < D; c += 8) {
        const uint4 q = *reinterpret_cast<const uint4*>(tot + c);
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int d0 = c + 2 * i;
            if (d0 < bestD - 1 || d0 > bestD + 1) alt = imin(alt, (int)(int16_t)(w[i] & 0xffff));
            if (d0 + 1 < bestD - 1 || d0 + 1 > bestD + 1) alt = imin(alt, (int)(int16_t)(w[i] >> 16));
        }
    }
    const int c0 = bestD > 0 ? (int)tot[bestD - 1] : 0;
    const int c1 = tot[bestD];
    const int c2 = bestD + 1 < D ? (int)tot[bestD + 1] : 0;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    int16_t dout = inv;
    float cout = 0.0f;
    if constexpr (PYR) {
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
            if (x2 >= 0 && x2 < J.w) atomicMin(&keys[x2], disp2_key(minCost, x));
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
            if (x2 >= 0 && x2 < J.w) atomicMin(&keys[x2], disp2_key(minCost, x));
            const float den = fmaxf((float)minCost, 1.0f);
            cout = fminf(fmaxf(((float)alt - (float)minCost) / den, 0.0f), 1.0f);
        }
    }
    const size_t p = (size_t)y * J.w + x;
    J.disp_raw[p] = dout;
    J.conf_raw[p] = cout;
}

// ---------------------------------------------------------------------------
// Row kernel: L->R and R->L of one row, WTA, disp2, LR check.  One warp per
// block; each warp owns 32/G rows (one per lane group).  Per step both
// paths advance one pixel; their recurrences are issued back to back
// (independent dependency chains).  Inputs are prefetched kPF steps ahead.
// The first path to reach a pixel leaves its partial sum in V, except near
// the meeting point, where the second path arrives kPF steps later at most:
// those partials go through a small shared-memory band, so a prefetched V
// never predates the write it needs.  The path that finishes a pixel stashes
// the pixel's D total costs in a shared buffer; every G steps each lane
// finishes one stashed pixel (argmin, second minimum, uniqueness,
// confidence, sub-pixel, disp2) and the G results are written together.
// ---------------------------------------------------------------------------
template <int G, int K, bool PYR, int NJ>
__global__ void __launch_bounds__(32) k_path_row(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.y];
    constexpr int RPW = 32 / G;
    constexpr int kPF = pf_depth<K>();
    constexpr int NB = kPF + 2;
    constexpr int DP = G * K;     // labels including padding
    constexpr int WS = DP + 8;    // stash row stride (int16): 16-byte rows, spread over banks
    const int W = J.w, H = J.h, D = J.D;
    const int y0 = blockIdx.x * RPW;
    if (y0 >= H) return;
    const int lane = threadIdx.x, gl = lane % G, grp = lane / G;
    const bool active = y0 + grp < H;
    const int y = active ? y0 + grp : H - 1;

    extern __shared__ __align__(16) unsigned char sm[];
    int* lut = reinterpret_cast<int*>(sm);
    unsigned char* sp = sm + 1024;
    int16_t* stash = reinterpret_cast<int16_t*>(sp) + grp * (2 * G * WS);  // [path][slot][WS]
    sp += (size_t)RPW * 2 * G * WS * 2;
    int16_t* band = reinterpret_cast<int16_t*>(sp) + grp * (NB * DP);
    sp += (size_t)RPW * NB * DP * 2;
    int16_t* xb = reinterpret_cast<int16_t*>(sp) + grp * (4 * DP);
    sp += (K > 1 ? (size_t)RPW * 4 * DP * 2 : 0);
    unsigned* keys = reinterpret_cast<unsigned*>(sp) + grp * W;
    if (J.adaptive)
        for (int i = lane; i < 256; i += 32) lut[i] = J.p2lut[i];
    for (int x = gl; x < W; x += G) keys[x] = kNoKey;
    __syncwarp();

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
    // a pixel x covered by both paths is reached |2x - C2| steps apart
    const int C2 = W - 1 + lr_x0;
    const int band_lo = (C2 - kPF + 1) >> 1;
    auto in_band = [&](int x) { return abs(2 * x - C2) <= kPF; };
    auto rl_covers = [&](int x) { return x >= W - rl_n; };
    auto lr_covers = [&](int x) { return lr_n > 0 && x >= lr_x0 && x < lr_x0 + lr_n; };
    auto wta_px = [&](int x) { return PYR || (x >= minX1 && x < maxX1 && x != W - 1); };
    auto pf_lr = [&](int s, Pre<K>& f) {
        if (s < lr_n) prefetch<K, PYR>(J, y, lr_x0 + s, gl, true, f);
    };
    auto pf_rl = [&](int s, Pre<K>& f) {
        if (s < rl_n) prefetch<K, PYR>(J, y, W - 1 - s, gl, true, f);
    };
    // first arrival: fold in T->B, leave the partial in the band or in V
    auto leave = [&](int x, const int (&L)[K], const int (&vin)[K]) {
        int part[K];
        combine_first<K, PYR>(L, vin, has_tb, part);
        if (in_band(x)) {
            int16_t* b = band + (x - band_lo) * DP + gl * K;
#pragma unroll
            for (int k = 0; k < K; ++k) b[k] = (int16_t)part[k];
        } else if (active && PG_IN(((size_t)y * W + x) * D, D, (size_t)W * H * D, 13)) {
            store_labels<K>(J.V + ((size_t)y * W + x) * D, D, gl, part);
        }
    };
    // second arrival: the total of all paths
    auto total = [&](int x, const int (&L)[K], const int (&vin)[K], int (&tot)[K]) {
        int part[K];
        if (in_band(x)) {
            const int16_t* b = band + (x - band_lo) * DP + gl * K;
#pragma unroll
            for (int k = 0; k < K; ++k) part[k] = b[k];
        } else {
#pragma unroll
            for (int k = 0; k < K; ++k) part[k] = vin[k];
        }
        combine_second<K, PYR>(part, L, tot);
        if (J.debug_acc && active) store_labels<K>(J.V + ((size_t)y * W + x) * D, D, gl, tot);
    };
    // deferred WTA: slot `slot` of path `path` holds pixel wx[path] of lane `slot`
    int wx[2] = {-1, -1}, wbase[2] = {0, 0}, wvc[2] = {0, 0};
    auto stash_px = [&](int path, int slot, int x, const int (&tot)[K], const StepIn<K>& in) {
        int16_t* s = stash + (path * G + slot) * WS + gl * K;
#pragma unroll
        for (int k = 0; k < K; ++k) s[k] = (int16_t)tot[k];
        if (gl == slot) {
            wx[path] = x;
            wbase[path] = in.base;
            wvc[path] = in.vc;
        }
    };
    auto flush = [&]() {
        __syncwarp();
#pragma unroll
        for (int path = 0; path < 2; ++path) {
            if (wx[path] >= 0 && active)
                finish_pixel<PYR>(J, y, wx[path], stash + (path * G + gl) * WS, wbase[path], wvc[path], keys);
            wx[path] = -1;
        }
        __syncwarp();
    };

    Chain<K> lr, rl;
    chain_init(lr, J.minD);
    chain_init(rl, J.minD);
    // Value-initialised: without an L->R path (numPaths == 1) its ring is never
    // loaded, yet its recurrence still runs (idle) beside the R->L one.
    Pre<K> plr[kPF] = {}, prl[kPF] = {};
#pragma unroll
    for (int j = 0; j < kPF; ++j) {
        pf_lr(j, plr[j]);
        pf_rl(j, prl[j]);
    }
    int lr_img_prev = 0, rl_img_prev = 0;
    const bool has_lr = lr_n > 0;
    const int T = imax(lr_n, rl_n);
    for (int t0 = 0; t0 < T; t0 += kPF) {
#pragma unroll
        for (int j = 0; j < kPF; ++j) {
            const int t = t0 + j;
            if (t < T) {
                const int xl = lr_x0 + imin(t, imax(lr_n - 1, 0));
                const int xr = W - 1 - imin(t, rl_n - 1);
                StepIn<K> il, ir;
                make_step<K, PYR>(J, xl, gl, plr[j], il);
                make_step<K, PYR>(J, xr, gl, prl[j], ir);
                il.p2 = (J.adaptive && lr.active) ? lut[abs(plr[j].img - lr_img_prev) & 255] : J.P2;
                ir.p2 = (J.adaptive && rl.active) ? lut[abs(prl[j].img - rl_img_prev) & 255] : J.P2;
                lr_img_prev = plr[j].img;
                rl_img_prev = prl[j].img;
                int vl[K], vr[K];
#pragma unroll
                for (int k = 0; k < K; ++k) { vl[k] = plr[j].v[k]; vr[k] = prl[j].v[k]; }
                pf_lr(t + kPF, plr[j]);
                pf_rl(t + kPF, prl[j]);
                // both recurrences back to back (a finished L->R path only idles)
                int Ll[K], Lr[K];
                chain_step<G, K, PYR>(lr, il, J.P1, D, gl, xb, Ll);
                chain_step<G, K, PYR>(rl, ir, J.P1, D, gl, xb + 2 * DP, Lr);
                const int slot = t & (G - 1);
                if (has_lr && t < lr_n && rl_covers(xl)) {
                    if ((W - 1 - xl) < t) {
                        int tot[K];
                        total(xl, Ll, vl, tot);
                        if (wta_px(xl)) stash_px(0, slot, xl, tot, il);
                    } else {
                        leave(xl, Ll, vl);
                    }
                }
                if (t < rl_n) {
                    if (!has_lr) {
                        // R->L is the only horizontal path (and there is no T->B)
                        if (J.debug_acc && active) store_labels<K>(J.V + ((size_t)y * W + xr) * D, D, gl, Lr);
                        if (wta_px(xr)) stash_px(1, slot, xr, Lr, ir);
                    } else if (lr_covers(xr)) {
                        if ((xr - lr_x0) <= t) {
                            int tot[K];
                            total(xr, Lr, vr, tot);
                            if (wta_px(xr)) stash_px(1, slot, xr, tot, ir);
                        } else {
                            leave(xr, Lr, vr);
                        }
                    }
                }
                if (slot == G - 1 || t == T - 1) flush();
            }
        }
    }

    // LR check over the finished row and the final per-pixel write.
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    const bool check = (J.post & POST_LRCHECK) != 0;
    for (int x = gl; x < W; x += G) {
        const size_t pp = (size_t)y * W + x;
        const bool wp = wta_px(x);
        int d16 = inv;
        float cf = 0.0f;
        if (wp) { d16 = J.disp_raw[pp]; cf = J.conf_raw[pp]; }
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
        if (active) { J.disp_raw[pp] = (int16_t)d16; J.conf_raw[pp] = cf; }
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
        if ((err = launched(st, "k_path_tb")) != cudaSuccess) return err;
    }
    constexpr int RPW = 32 / G;
    constexpr int DP = G * K;
    const size_t smem = 1024 + (size_t)RPW * 2 * G * (DP + 8) * 2 + (size_t)RPW * (pf_depth<K>() + 2) * DP * 2 +
                        (K > 1 ? (size_t)RPW * 4 * DP * 2 : 0) + (size_t)RPW * e.max_w * 4;
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
    return launched(st, "k_path_row");
}

// Words per thread of the packed kernels for a launch: 8 (one thread per
// 16-label chain, the fewest instructions per pixel) when the launch has
// rows enough for one such warp per SM, else the shorter-step shape
// (2 words, or 4 for 64 labels).  packed_words_override() (set through
// pyrsgm_gb300_set_packed_words) forces one of them.
inline int packed_nw(int D, long long rows)
{
    const int force = packed_words_override();
    const int small = D == 64 ? 4 : 2;
    if (force == 8) return 8;
    if (force == 2 || force == 4) return small;
    const long long warps8 = rows * 2 * (D / 16) / 32;
    return warps8 >= (long long)packed_min_warps_per_sm() * sm_count() ? 8 : small;
}

// Words per thread for a packed launch: a forced setting, else a recorded
// measurement for its key, else (measuring it now when the thread is in a
// tuning scope) the rule of packed_nw().  `run(nw)` launches one shape.
template <class Run>
int packed_choice(const TuneKey& key, long long rows, cudaStream_t st, Run run, cudaError_t& err)
{
    err = cudaSuccess;
    if (packed_words_override() != 0 || !autotune_enabled()) return packed_nw(key.D, rows);
    TuneEntry te;
    if (tune_lookup(key, te)) return te.nw;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (!tuning_thread() || cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return packed_nw(key.D, rows);
    const int spread = key.D == 64 ? 4 : 2;
    float best[2] = {1e30f, 1e30f};
    cudaEvent_t a = nullptr, b = nullptr;
    if ((err = cudaEventCreate(&a)) != cudaSuccess || (err = cudaEventCreate(&b)) != cudaSuccess) {
        if (a) cudaEventDestroy(a);
        return packed_nw(key.D, rows);
    }
    for (int rep = 0; rep < 2 && err == cudaSuccess; ++rep) {
        for (int c = 0; c < 2 && err == cudaSuccess; ++c) {
            float ms = 0.0f;
            if ((err = cudaEventRecord(a, st)) != cudaSuccess || (err = run(c == 0 ? 8 : spread)) != cudaSuccess ||
                (err = cudaEventRecord(b, st)) != cudaSuccess || (err = cudaEventSynchronize(b)) != cudaSuccess ||
                (err = cudaEventElapsedTime(&ms, a, b)) != cudaSuccess)
                break;
            best[c] = std::min(best[c], ms);
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (err != cudaSuccess) return packed_nw(key.D, rows);
    te.nw = best[0] <= best[1] ? 8 : spread;
    te.ms_wide = best[0];
    te.ms_spread = best[1];
    tune_store(key, te);
    return te.nw;
}

template <bool PYR, int NJ>
cudaError_t launch_paths_mode(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    long long rows = 0;
    for (int i = 0; i < jobs.n; ++i) rows += jobs.d[i].h;
    const int D = jobs.d[0].D;
    // 16-label pyramid levels with all three paths: the wide shape is the
    // fused T->B + L->R and R->L + WTA passes (k_fused.cuh)
    bool fused = false;
    if constexpr (PYR) fused = D == 16 && fused_mode() != 0 && fused_applicable(jobs);
    const TuneKey key{D, PYR ? (fused ? 2 : D == 16 && tbw_mode() ? 3 : 1) : 0, (int)std::min<long long>(rows, INT_MAX), e.max_w};
    cudaError_t err = cudaSuccess;
    switch (path_variant(D)) {
    case 10016: {
        auto run = [&](int nw) {
            if constexpr (PYR) {
                if (nw == 8 && fused) return launch_paths_fused16<NJ>(jobs, e, st);
            }
            return nw == 8 ? launch_paths_packed<8, 1, PYR, NJ>(jobs, e, st)
                           : launch_paths_packed<2, 4, PYR, NJ>(jobs, e, st);
        };
        const int nw = packed_choice(key, rows, st, run, err);
        return err != cudaSuccess ? err : run(nw);
    }
    case 10032: {
        auto run = [&](int nw) {
            return nw == 8 ? launch_paths_packed<8, 2, PYR, NJ>(jobs, e, st)
                           : launch_paths_packed<2, 8, PYR, NJ>(jobs, e, st);
        };
        const int nw = packed_choice(key, rows, st, run, err);
        return err != cudaSuccess ? err : run(nw);
    }
    case 10064: {
        auto run = [&](int nw) {
            return nw == 8 ? launch_paths_packed<8, 4, PYR, NJ>(jobs, e, st)
                           : launch_paths_packed<4, 8, PYR, NJ>(jobs, e, st);
        };
        const int nw = packed_choice(key, rows, st, run, err);
        return err != cudaSuccess ? err : run(nw);
    }
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
