// k_paths_packed.cuh -- path aggregation for D = 2*NW*T labels (16, 32,
// 64): the labels of one path chain are packed two per 32-bit word and held
// by T threads, NW words each.  NW = 8 (a 16-label chain is one thread)
// spends the fewest instructions per pixel and suits launches with many
// rows; NW = 2 spreads a chain over more threads, shortening each step, for
// launches with few rows (one pair, coarse levels).
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
// Shifted windows: each step a thread stores its NW words of the
// previous step into its chain's guard-padded shared buffer and reads back
// the NW + 2 words of its shifted window (word w of chain c at w * CPW + c, so
// a one-thread chain touches only its own bank).  Chains of T > 1 threads
// double-buffer the window and exchange it with one __syncwarp per step;
// their minima reduce by __shfl_xor_sync.
//
// Loads: rings in shared memory filled with cp.async, so the loads of a
// step are issued several steps before it without holding registers.  The
// T->B pass has one slot per step and thread (a warp's 32 columns are
// adjacent, so its requests are whole lines already); the horizontal pass
// of the NW = 8 shapes moves 128-byte runs of each chain with the whole
// warp (chunk_steps), that of the spread shapes streams per lane.
//
// Paths: the T->B chains write their costs into V, the L->R and R->L chains
// of each row into Vl and Vr; the chains never exchange data.  The WTA
// kernel adds the three (one cap and one sentinel make the clamped sum
// order-free), picks the winner and writes the disp2 candidates to the
// per-pixel keys with atomicMin; the LR check reads them in the post kernel.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {

namespace pk {

constexpr uint32_t kMax2 = 0x7fff7fffu;
constexpr uint32_t kOne2 = 0x00010001u;
// Warps per block: 4 for the one-thread-per-16-labels shape (throughput on
// many rows), 2 for the spread shapes (more, smaller blocks for few rows).
template <int NW>
__host__ __device__ constexpr int warps_of() { return NW == 8 ? 4 : 2; }
constexpr int kStagesTb = 8;     // look-ahead of the top->bottom pass
constexpr int kStagesLane = 6;   // look-ahead of the per-lane horizontal pass

__device__ __forceinline__ uint32_t dup(int v) { return ((uint32_t)v & 0xffffu) * 0x10001u; }

// 0xffff in each 16-bit half whose bit 15 is set, else 0.
__device__ __forceinline__ uint32_t sign_mask2(uint32_t x)
{
    uint32_t r;
    asm("prmt.b32 %0, %1, 0, 0xBB99;" : "=r"(r) : "r"(x));
    return r;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp16(void* dst, const void* src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp8(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp4(void* dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// The aligned 32-bit word holding the byte at p (it lies in the same
// allocation as the byte).
__device__ __forceinline__ const void* word_of(const void* p)
{
    return reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)3);
}
__device__ __forceinline__ int byte_shift(const void* p) { return (int)(reinterpret_cast<uintptr_t>(p) & 3) * 8; }

template <int NW, int T>
struct Grp {
    static constexpr int D = 2 * NW * T;        // labels per chain
    static constexpr int CPW = 32 / T;          // chains per warp
    static constexpr int PADW = D / 2 + 1;      // guard words before label 0 (D + 2 halves)
    static constexpr int LENW = PADW + D + 2;   // words a shifted window can touch
    static constexpr int BUFW = LENW * CPW;     // one window buffer of a warp
    static constexpr int NBUF = T == 1 ? 1 : 2;
    // Ring slot of a thread: its NW cost words.  For NW = 8 the two 16-byte
    // halves of a slot are swapped in lanes 4-7 of every 8 (ring_half), so
    // that the 16-byte accesses of 8 lanes at a 32-byte stride hit distinct
    // banks.  The label-base and image words of a slot sit in a separate
    // [slot][2][32] array (bank = lane).
    static constexpr int RSW_TB = NW;
};

template <int NW>
struct GChain {
    uint32_t L[NW];
    int mp;        // minimum of the previous step over the chain's labels
    int prevBase;
};

template <int NW>
__device__ __forceinline__ void gchain_init(GChain<NW>& s, int minD)
{
#pragma unroll
    for (int i = 0; i < NW; ++i) s.L[i] = kMax2;
    s.mp = 0x7fff;
    s.prevBase = minD;
}

// NW consecutive words (16-byte aligned for NW >= 4, 8-byte for NW == 2).
template <int NW>
__device__ __forceinline__ void ldw(const uint32_t* p, uint32_t (&v)[NW])
{
    if constexpr (NW == 2) {
        const uint2 a = *reinterpret_cast<const uint2*>(p);
        v[0] = a.x; v[1] = a.y;
    } else {
#pragma unroll
        for (int i = 0; i < NW / 4; ++i) {
            const uint4 a = reinterpret_cast<const uint4*>(p)[i];
            v[4 * i] = a.x; v[4 * i + 1] = a.y; v[4 * i + 2] = a.z; v[4 * i + 3] = a.w;
        }
    }
}
template <int NW>
__device__ __forceinline__ void stw(uint32_t* p, const uint32_t (&v)[NW])
{
    if constexpr (NW == 2) {
        *reinterpret_cast<uint2*>(p) = make_uint2(v[0], v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < NW / 4; ++i)
            reinterpret_cast<uint4*>(p)[i] = make_uint4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    }
}
// Asynchronous copy of NW words.
template <int NW>
__device__ __forceinline__ void cpw(uint32_t* dst, const int16_t* src)
{
    if constexpr (NW == 2) {
        cp8(dst, src);
    } else {
#pragma unroll
        for (int i = 0; i < NW / 4; ++i) cp16(dst + 4 * i, src + 8 * i);
    }
}

// Position of half h (0, 1) of an NW = 8 ring slot in lane `lane`'s slot.
__device__ __forceinline__ int ring_half(int h, int lane) { return 4 * (h ^ ((lane >> 2) & 1)); }

// Minimum over the chain's words: a tree in the thread, then over the group.
template <int NW, int T>
__device__ __forceinline__ uint32_t chain_min2(const uint32_t (&L)[NW])
{
    uint32_t m2;
    if constexpr (NW == 2) {
        m2 = __vminu2(L[0], L[1]);
    } else if constexpr (NW == 4) {
        m2 = __vimin3_u16x2(L[0], L[1], __vminu2(L[2], L[3]));
    } else {
        m2 = __vminu2(__vimin3_u16x2(L[0], L[1], L[2]), __vimin3_u16x2(L[3], L[4], L[5]));
        m2 = __vimin3_u16x2(m2, L[6], L[7]);
    }
#pragma unroll
    for (int o = 1; o < T; o <<= 1) m2 = __vminu2(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    return m2;
}

// One step of the chain: c = this thread's 2*NW costs of the pixel,
// buf = word 0 of the chain's window buffer (this step's parity).
template <int NW, int T, bool PYR>
__device__ __forceinline__ void gstep(GChain<NW>& s, const uint32_t (&c)[NW], int base, int p2, uint32_t p12,
                                      uint32_t* buf, int k)
{
    using G = Grp<NW, T>;
    constexpr int D = G::D, ST = G::CPW;
#pragma unroll
    for (int i = 0; i < NW; ++i) buf[(G::PADW + NW * k + i) * ST] = s.L[i];
    if (T > 1) __syncwarp();
    int delta = PYR ? base - s.prevBase : 0;
    delta = iclamp(delta, -(D + 1), D + 1);
    const int i0 = 2 * G::PADW + delta - 1 + 2 * NW * k;   // half index of label (2NW*k - 1) after the shift
    const uint32_t* wp = buf + (i0 >> 1) * ST;
    const uint32_t sh = (uint32_t)(i0 & 1) * 16;
    uint32_t w0[NW + 2];
#pragma unroll
    for (int j = 0; j < NW + 2; ++j) w0[j] = wp[j * ST];
    uint32_t w[NW + 1];
#pragma unroll
    for (int j = 0; j < NW + 1; ++j) w[j] = __funnelshift_r(w0[j], w0[j + 1], sh);
    const int lj = imin(0x7fff, s.mp + p2);
    const uint32_t lj2 = dup(lj), mp2 = dup(s.mp);
    const uint32_t inc2 = (PYR && s.mp < 0x7fff) ? kOne2 : 0u;
#pragma unroll
    for (int m = 0; m < NW; ++m) {
        const uint32_t n0 = __funnelshift_r(w[m], w[m + 1], 16);   // (L[s], L[s+1])
        const uint32_t t = __viaddmin_u16x2(w[m], p12, lj2);       // min(L[s-1] + P1, lj)
        const uint32_t best = __vimin3_u16x2(n0, t, w[m + 1] + p12);
        uint32_t v = __viaddmin_u16x2(c[m], best - mp2, kMax2);
        if constexpr (PYR) v |= sign_mask2(best + inc2) & kMax2;
        s.L[m] = v;
    }
    const uint32_t m2 = chain_min2<NW, T>(s.L);
    s.mp = imin((int)(m2 & 0xffffu), (int)(m2 >> 16));
    s.prevBase = base;
}

// Coarse pyramid levels: labels outside label_range take SHRT_MAX.
template <int NW>
__device__ __forceinline__ void mask_labels(uint32_t (&c)[NW], int lo, int hi, int k)
{
    const int d0 = 2 * NW * k;
    if (lo <= d0 && hi >= d0 + 2 * NW - 1) return;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
        const int d = d0 + 2 * i;
        const bool ok0 = d >= lo && d <= hi, ok1 = d + 1 >= lo && d + 1 <= hi;
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

// Three-path total of one word (labels 2i, 2i+1) at a pyramid level: the
// sum clamped at SHRT_MAX - 1, SHRT_MAX where any path is SHRT_MAX -- the
// same as two gcombine<true>, in seven instructions instead of fourteen.
__device__ __forceinline__ uint32_t gtotal3(uint32_t a, uint32_t b, uint32_t c)
{
    const uint32_t s = __viaddmin_u16x2(__viaddmin_u16x2(b, c, 0x7ffe7ffeu), a, 0x7ffe7ffeu);
    return s | (sign_mask2(__vimax3_u16x2(a, b, c) + kOne2) & kMax2);
}

// Half j (0..15, not a compile-time constant) of 8 packed words, by a
// select tree on the bits of j: no indexed access, so the words stay in
// registers.
__device__ __forceinline__ int half_of(const uint32_t (&t)[8], int j)
{
    const bool b1 = j & 2, b2 = j & 4, b3 = j & 8;
    const uint32_t p0 = b1 ? t[1] : t[0], p1 = b1 ? t[3] : t[2], p2 = b1 ? t[5] : t[4], p3 = b1 ? t[7] : t[6];
    const uint32_t q0 = b2 ? p1 : p0, q1 = b2 ? p3 : p2;
    const uint32_t w = b3 ? q1 : q0;
    return (int)((w >> ((j & 1) * 16)) & 0xffffu);
}

// Winner over 16 packed labels, as k_wta defines it: minimum cost and the
// first label reaching it (minimum of the keys cost << 4 | label), the
// minimum cost over labels farther than one from it, and the costs next to
// it (0 outside the range).
__device__ __forceinline__ void wta16(const uint32_t (&t)[8], int& minCost, int& bestD, int& alt, int& c0, int& c2)
{
    uint32_t k[16];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        k[2 * i] = ((t[i] << 4) & 0xffff0u) | (uint32_t)(2 * i);
        k[2 * i + 1] = ((t[i] >> 12) & 0xffff0u) | (uint32_t)(2 * i + 1);
    }
    auto min16 = [](const uint32_t (&v)[16]) {
        const uint32_t a = __vimin3_u32(v[0], v[1], v[2]), b = __vimin3_u32(v[3], v[4], v[5]);
        const uint32_t c = __vimin3_u32(v[6], v[7], v[8]), d = __vimin3_u32(v[9], v[10], v[11]);
        const uint32_t e = __vimin3_u32(v[12], v[13], v[14]);
        const uint32_t x = __vimin3_u32(a, b, c), y = __vimin3_u32(d, e, v[15]);
        return x < y ? x : y;
    };
    const uint32_t best = min16(k);
    minCost = (int)(best >> 4);
    bestD = (int)(best & 15u);
    const int nb = 1 - bestD;
    uint32_t far[16];
#pragma unroll
    for (int d = 0; d < 16; ++d) far[d] = (unsigned)(d + nb) <= 2u ? 0xffffffffu : k[d];
    alt = (int)(min16(far) >> 4);
    c0 = bestD > 0 ? half_of(t, bestD - 1) : 0;
    c2 = bestD < 15 ? half_of(t, bestD + 1) : 0;
}

// Outputs of a winner (kernel_WTA_Subpixel, src/sgm_kernels.cu:573-640;
// pyramid kernel_PyramidWTA, src/sgm_kernels.cu:1290-1370): minimum cost,
// first label reaching it, the minimum over labels farther than one from
// it, and the costs next to it (c0, c2; 0 outside the range).
template <int D, bool PYR>
__device__ __forceinline__ void wta_out(const LevelDesc& J, int y, int x, int base, int minCost, int bestD, int alt,
                                        int c0, int c1, int c2)
{
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

// Horizontal pass I/O: CH steps of one chain are one 128-byte run of a
// cost or path volume (D = 16: 4 pixels, 32: 2, 64: 1).  The warp moves
// the runs of all its chains between global and shared memory together, 8
// lanes per run, so every request is a whole 128-byte line: one 32-byte
// stream per lane (a row and direction each) reaches about half the HBM
// bandwidth of line requests.  SC chunk slots in flight per warp.
template <int D>
__host__ __device__ constexpr int chunk_steps() { return D >= 64 ? 1 : 64 / D; }
// Chunk slots per warp (SC - 1 runs in flight): for 4-step runs 3 measured
// fastest on the 1080p row pass (2: too little look-ahead; 4: the larger
// footprint was slower as well); shorter runs keep about 6-8 steps of
// look-ahead.  A separate output chunk per warp (8 warps per SM) measured
// faster than writing the path costs back into the consumed slot with 12
// or 16 warps per SM (2.81 against 3.73 / 3.57 ms per 32-pair step).
template <int D>
__host__ __device__ constexpr int chunk_stages() { return chunk_steps<D>() == 4 ? 3 : chunk_steps<D>() == 2 ? 4 : 6; }

template <int NW, int T>
constexpr size_t row_smem()
{
    using G = Grp<NW, T>;
    constexpr int CH = chunk_steps<G::D>(), SC = chunk_stages<G::D>();
    // per warp: window buffers, SC input chunk slots and one output chunk
    // (32 words per chain each), the label-base / image ring
    return 256 * 4 + (size_t)warps_of<NW>() * 4 * (G::NBUF * G::BUFW + (SC + 1) * G::CPW * 32 + SC * CH * 64);
}
template <int NW, int T>
constexpr size_t row_lane_smem()
{
    using G = Grp<NW, T>;
    return 256 * 4 + (size_t)warps_of<NW>() * 4 * (G::NBUF * G::BUFW + kStagesLane * 32 * (G::RSW_TB + 2));
}
template <int NW, int T>
constexpr size_t tb_smem()
{
    using G = Grp<NW, T>;
    return 256 * 4 + (size_t)warps_of<NW>() * 4 * (G::NBUF * G::BUFW + kStagesTb * 32 * (G::RSW_TB + 2));
}

}  // namespace pk

// ---------------------------------------------------------------------------
// Top -> bottom: a warp holds 32/T adjacent columns, T threads each.
// ---------------------------------------------------------------------------
template <int NW, int T, bool PYR, int NJ>
__global__ void __launch_bounds__(pk::warps_of<NW>() * 32) k_gtb(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<NW, T>;
    constexpr int D = G::D, S = kStagesTb, RS = G::RSW_TB, kWarps = warps_of<NW>();
    const LevelDesc& J = jobs.d[blockIdx.y];
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    uint32_t* cbuf = smem + 256;
    uint32_t* rbuf = cbuf + kWarps * G::NBUF * G::BUFW;
    uint32_t* bibuf = rbuf + kWarps * S * 32 * RS;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * G::NBUF * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lane / T, k = lane % T;
    uint32_t* bi = bibuf + warp * S * 64 + lane;   // [slot][base, image][lane]
    int xlo = 0, xhi = J.w;
    if (!PYR) { xlo = imax(J.minD + D, 0); xhi = J.w + imin(J.minD, 0); }
    const int ncol = xhi - xlo;
    const int col0 = (blockIdx.x * kWarps + warp) * G::CPW;
    if (col0 >= ncol) return;   // the whole warp is past the image
    const int col = col0 + c;
    const bool col_ok = col < ncol;
    const int x = xlo + imin(col, ncol - 1), H = J.h, W = J.w;
    uint32_t* chain = cbuf + warp * G::NBUF * G::BUFW + c;
    uint32_t* ring = rbuf + (warp * S * 32 + lane) * RS;
    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    int lo = 0, hi = D - 1;
    if (PYR && !J.refine) label_range(J, x, J.minD, lo, hi);
    const bool use_base = PYR && J.refine, adaptive = J.adaptive != 0;
    const int16_t* const Cg = J.C;
    int16_t* const Vg = J.V;
    const int16_t* const Bg = J.base;
    const uint8_t* const Lg = J.left;
    const size_t vstep = (size_t)W * D, lstep = (size_t)J.lstep;
    // issue cursor (row yi) and consume cursor (row y)
    size_t oi = (size_t)x * D + 2 * NW * k, pi = x, li = x;
    size_t oc = oi, pc = pi, lc = li;
    int yi = 0;
    auto issue_next = [&](int slot) {
        if (yi < H && PG_IN(oi, 2 * NW, (size_t)W * H * D, 1)) {
            uint32_t* d = ring + slot * 32 * RS;
            if constexpr (NW == 8) {
                cp16(d + ring_half(0, lane), Cg + oi);
                cp16(d + ring_half(1, lane), Cg + oi + 8);
            } else {
                cpw<NW>(d, Cg + oi);
            }
            if (use_base) cp4(bi + slot * 64, word_of(Bg + pi));
            if (adaptive) cp4(bi + slot * 64 + 32, word_of(Lg + li));
        }
        cp_commit();
        ++yi;
        oi += vstep;
        pi += W;
        li += lstep;
    };
    GChain<NW> s;
    gchain_init(s, J.minD);
#pragma unroll
    for (int j = 0; j < S - 1; ++j) issue_next(j);
    int img_prev = 0, slot = 0, islot = S - 1;
#pragma unroll 2
    for (int y = 0; y < H; ++y) {
        issue_next(islot);
        islot = islot + 1 == S ? 0 : islot + 1;
        cp_wait<S - 1>();
        const uint32_t* d = ring + slot * 32 * RS;
        const uint32_t* db = bi + slot * 64;
        slot = slot + 1 == S ? 0 : slot + 1;
        uint32_t cc[NW];
        if constexpr (NW == 8) {
            const uint4 a = *reinterpret_cast<const uint4*>(d + ring_half(0, lane));
            const uint4 b = *reinterpret_cast<const uint4*>(d + ring_half(1, lane));
            cc[0] = a.x; cc[1] = a.y; cc[2] = a.z; cc[3] = a.w;
            cc[4] = b.x; cc[5] = b.y; cc[6] = b.z; cc[7] = b.w;
        } else {
            ldw<NW>(d, cc);
        }
        const int base = use_base ? (int)(int16_t)(db[0] >> ((pc & 1) * 16)) : J.minD;
        int p2 = J.P2;
        if (adaptive) {
            const int img = (int)((db[32] >> byte_shift(Lg + lc)) & 255u);
            p2 = lut[abs(img - img_prev) & 255];
            img_prev = img;
        }
        if (PYR && !J.refine) mask_labels<NW>(cc, lo, hi, k);
        gstep<NW, T, PYR>(s, cc, base, p2, p12, chain + (G::NBUF == 2 ? (y & 1) * G::BUFW : 0), k);
        if (col_ok && PG_IN(oc, 2 * NW, (size_t)W * H * D, 2)) stw<NW>(reinterpret_cast<uint32_t*>(Vg + oc), s.L);
        oc += vstep;
        pc += W;
        lc += lstep;
    }
    cp_wait<0>();
}

// ---------------------------------------------------------------------------
// Horizontal paths: a warp holds 16/T rows, each with an L->R chain group
// and an R->L chain group of T threads.  Each chain walks its whole range
// and stores its path costs (L->R into Vl, R->L into Vr); the chains of a
// row never exchange data, and the WTA kernel adds the paths.
//
// Costs come in and path costs go out in chunks of CH steps per chain (one
// 128-byte run each, chunk_steps): lane l of the warp moves 16-byte piece
// l % 8 of the runs of chains 4j + l / 8 (j < CPW / 4), which all share one
// direction ((l / 8) & 1) and so one step -> x mapping.  A chain's run sits
// in 32 shared words with piece p at column p ^ (chain & 7), so that both
// the line-wide copies and the per-chain reads of a step are free of bank
// conflicts.
// ---------------------------------------------------------------------------
template <int NW, int T, bool PYR, int NJ>
__global__ void __launch_bounds__(pk::warps_of<NW>() * 32) k_grow(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<NW, T>;
    constexpr int D = G::D, CPW = G::CPW, RPW = CPW / 2, kWarps = warps_of<NW>();
    constexpr int CH = chunk_steps<D>(), SC = chunk_stages<D>();
    constexpr int PPX = D / 8;          // 16-byte pieces per pixel
    constexpr int NCOP = CPW / 4;       // pieces a lane moves per chunk
    constexpr int SLOTW = CPW * 32;     // words of one chunk slot
    const LevelDesc& J = jobs.d[blockIdx.y];
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    uint32_t* cbuf = smem + 256;
    uint32_t* rbuf = cbuf + kWarps * G::NBUF * G::BUFW;
    uint32_t* bibuf = rbuf + kWarps * (SC + 1) * SLOTW;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * G::NBUF * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lane / T, k = lane % T, r = c >> 1, dir = c & 1;
    const int row0 = (blockIdx.x * kWarps + warp) * RPW;
    if (row0 >= J.h) return;   // the whole warp is past the image
    const int y = row0 + r;
    const int yy = imin(y, J.h - 1);
    const int W = J.w, H = J.h;
    uint32_t* chain = cbuf + warp * G::NBUF * G::BUFW + c;
    uint32_t* ring = rbuf + warp * (SC + 1) * SLOTW;
    uint32_t* ob = ring + SC * SLOTW;
    uint32_t* bi = bibuf + warp * SC * CH * 64 + lane;   // [slot][2 * CH words][lane]

    // path extents (single-scale: kernel_AggregateLR/RL ranges)
    int lr_x0 = 0, lr_n, rl_n;
    if (PYR) {
        lr_n = J.paths >= 2 ? W : 0;
        rl_n = W;
    } else {
        const int minX1 = imax(J.minD + D, 0), maxX1 = W + imin(J.minD, 0);
        lr_x0 = minX1;
        lr_n = J.paths >= 2 ? imax(0, maxX1 - minX1) : 0;
        rl_n = imax(0, W - minX1);
    }
    const int Tn = imax(lr_n, rl_n);
    const int n_mine = dir == 0 ? lr_n : rl_n;
    const int dx = dir == 0 ? 1 : -1;
    const int xs = dir == 0 ? lr_x0 : W - 1;   // step t of a chain is at x = xs + dx * t
    const int16_t* const Cg = J.C;
    const int16_t* const Bg = J.base;
    const uint8_t* const Lg = J.left;
    const bool use_base = PYR && J.refine, adaptive = J.adaptive != 0;
    const int P2c = J.P2, minD = J.minD;
    const size_t prow = (size_t)yy * W, lrow = (size_t)yy * J.lstep;

    // this lane's share of the warp-wide chunk copies
    const int pce = lane & 7, cdir = (lane >> 3) & 1, crow = row0 + (lane >> 4);
    const int cq = pce / PPX, cs = cdir ? CH - 1 - cq : cq;   // pixel of the run, step of that pixel
    const int cn = cdir ? rl_n : lr_n, cxs = cdir ? W - 1 : lr_x0, cdx = cdir ? -1 : 1;
    const int coff = (pce % PPX) * 8;                          // int16 offset inside the pixel
    int16_t* const Og = cdir ? J.Vr : J.Vl;
    const size_t rstride = (size_t)2 * W * D;                  // two rows (chain 4j -> 4j + 4)
    auto piece_col = [](int chn, int p) { return chn * 32 + ((p ^ (chn & 7)) << 2); };

    int ci_issue = 0;
    auto issue_next = [&](int slot) {
        const int t = ci_issue * CH + cs;
        if (t < cn) {
            const size_t src = ((size_t)crow * W + (cxs + cdx * t)) * D + coff;
#pragma unroll
            for (int j = 0; j < NCOP; ++j)
                if (crow + 2 * j < H && PG_IN(src + j * rstride, 8, (size_t)W * H * D, 3))
                    cp16(ring + slot * SLOTW + piece_col(4 * j + (lane >> 3), pce), Cg + src + j * rstride);
        }
        // label bases and image bytes of this lane's own chain: [2 * CH][32]
        // words per slot, bases first.  A whole 4-step run whose bases sit
        // on a 4-byte boundary takes two word copies (pixel pairs), its
        // image bytes one; otherwise each step copies the word holding it.
        uint32_t* bslot = bi + slot * CH * 64;
        const int t0 = ci_issue * CH, xlo = dir ? xs - t0 - (CH - 1) : xs + t0;
        const bool full = CH == 4 && t0 + CH - 1 < n_mine;
        const bool fb = full && (reinterpret_cast<uintptr_t>(Bg + prow + xlo) & 3) == 0;
        const bool fi = full && (reinterpret_cast<uintptr_t>(Lg + lrow + xlo) & 3) == 0;
        if (use_base && fb) {
            cp4(bslot, Bg + prow + xlo);
            cp4(bslot + 32, Bg + prow + xlo + 2);
        }
        if (adaptive && fi) cp4(bslot + CH * 32, Lg + lrow + xlo);
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            const int ts = t0 + s;
            if (ts < n_mine) {
                const int x = xs + dx * ts;
                if (use_base && !fb) cp4(bslot + s * 32, word_of(Bg + prow + x));
                if (adaptive && !fi) cp4(bslot + (CH + s) * 32, word_of(Lg + lrow + x));
            }
        }
        cp_commit();
        ++ci_issue;
    };

    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    GChain<NW> st;
    gchain_init(st, minD);
    const int NC = (Tn + CH - 1) / CH;
#pragma unroll
    for (int j = 0; j < SC - 1; ++j) issue_next(j);
    int img_prev = 0, slot = 0, islot = SC - 1;
    for (int ci = 0; ci < NC; ++ci) {
        issue_next(islot);
        islot = islot + 1 == SC ? 0 : islot + 1;
        cp_wait<SC - 1>();
        __syncwarp();
        const uint32_t* cin = ring + slot * SLOTW;
        const uint32_t* db = bi + slot * CH * 64;
        const int t0 = ci * CH, xlo = dir ? xs - t0 - (CH - 1) : xs + t0;
        const bool full = CH == 4 && t0 + CH - 1 < n_mine;
        const bool fb = full && (reinterpret_cast<uintptr_t>(Bg + prow + xlo) & 3) == 0;
        const bool fi = full && (reinterpret_cast<uintptr_t>(Lg + lrow + xlo) & 3) == 0;
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            const int t = ci * CH + s;
            if (t >= Tn) break;   // the same for the whole warp
            // this lane's NW words of step s: word q * D / 2 + k * NW of the run
            const int q = dir ? CH - 1 - s : s;
            const int w0 = q * (D / 2) + k * NW;
            uint32_t cc[NW];
            if constexpr (NW == 2) {
                const uint2 a = *reinterpret_cast<const uint2*>(cin + piece_col(c, w0 >> 2) + (w0 & 3));
                cc[0] = a.x; cc[1] = a.y;
            } else {
#pragma unroll
                for (int i = 0; i < NW / 4; ++i) {
                    const uint4 a = *reinterpret_cast<const uint4*>(cin + piece_col(c, (w0 >> 2) + i));
                    cc[4 * i] = a.x; cc[4 * i + 1] = a.y; cc[4 * i + 2] = a.z; cc[4 * i + 3] = a.w;
                }
            }
            const int x = xs + dx * t;
            int base = minD;
            if (use_base)
                base = fb ? (int)(int16_t)(db[(q >> 1) * 32] >> ((q & 1) * 16))
                          : (int)(int16_t)(db[s * 32] >> (((prow + x) & 1) * 16));
            int p2 = P2c;
            if (adaptive) {
                const int img = fi ? (int)((db[CH * 32] >> (q * 8)) & 255u)
                                   : (int)((db[(CH + s) * 32] >> byte_shift(Lg + lrow + x)) & 255u);
                p2 = lut[abs(img - img_prev) & 255];
                img_prev = img;
            }
            if (PYR && !J.refine) {
                int lo, hi;
                label_range(J, x, minD, lo, hi);
                mask_labels<NW>(cc, lo, hi, k);
            }
            gstep<NW, T, PYR>(st, cc, base, p2, p12, chain + (G::NBUF == 2 ? (t & 1) * G::BUFW : 0), k);
            if constexpr (NW == 2) {
                *reinterpret_cast<uint2*>(ob + piece_col(c, w0 >> 2) + (w0 & 3)) = make_uint2(st.L[0], st.L[1]);
            } else {
#pragma unroll
                for (int i = 0; i < NW / 4; ++i)
                    *reinterpret_cast<uint4*>(ob + piece_col(c, (w0 >> 2) + i)) =
                        make_uint4(st.L[4 * i], st.L[4 * i + 1], st.L[4 * i + 2], st.L[4 * i + 3]);
            }
        }
        __syncwarp();
        {
            const int t = ci * CH + cs;
            if (t < cn) {
                const size_t dst = ((size_t)crow * W + (cxs + cdx * t)) * D + coff;
#pragma unroll
                for (int j = 0; j < NCOP; ++j)
                    if (crow + 2 * j < H && PG_IN(dst + j * rstride, 8, (size_t)W * H * D, 4))
                        *reinterpret_cast<uint4*>(Og + dst + j * rstride) =
                            *reinterpret_cast<const uint4*>(ob + piece_col(4 * j + (lane >> 3), pce));
            }
        }
        __syncwarp();
        slot = slot + 1 == SC ? 0 : slot + 1;
    }
    cp_wait<0>();
}

// ---------------------------------------------------------------------------
// Horizontal paths, per-lane loads: the same chains as k_grow, each thread
// streaming its own costs through a ring of kStagesLane steps and storing
// its path costs directly.  For the spread shapes (NW < 8) on launches with
// few rows, where the per-step latency of a chain bounds the pass rather
// than HBM: the warp-wide chunk copies of k_grow add two warp
// synchronisations and a shared-memory round trip to every chunk.
// ---------------------------------------------------------------------------
template <int NW, int T, bool PYR, int NJ>
__global__ void __launch_bounds__(pk::warps_of<NW>() * 32) k_grow_lane(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<NW, T>;
    constexpr int D = G::D, RPW = G::CPW / 2, S = kStagesLane, RS = G::RSW_TB, kWarps = warps_of<NW>();
    const LevelDesc& J = jobs.d[blockIdx.y];
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    uint32_t* cbuf = smem + 256;
    uint32_t* rbuf = cbuf + kWarps * G::NBUF * G::BUFW;
    uint32_t* bibuf = rbuf + kWarps * S * 32 * RS;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * G::NBUF * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = lane / T, k = lane % T, r = c >> 1, dir = c & 1;
    const int row0 = (blockIdx.x * kWarps + warp) * RPW;
    if (row0 >= J.h) return;   // the whole warp is past the image
    const int y = row0 + r;
    const bool row_ok = y < J.h;
    const int yy = imin(y, J.h - 1);
    const int W = J.w;
    uint32_t* chain = cbuf + warp * G::NBUF * G::BUFW + c;
    uint32_t* ring = rbuf + (warp * S * 32 + lane) * RS;
    uint32_t* bi = bibuf + warp * S * 64 + lane;   // [slot][base, image][lane]

    // path extents (single-scale: kernel_AggregateLR/RL ranges)
    int lr_x0 = 0, lr_n, rl_n;
    if (PYR) {
        lr_n = J.paths >= 2 ? W : 0;
        rl_n = W;
    } else {
        const int minX1 = imax(J.minD + D, 0), maxX1 = W + imin(J.minD, 0);
        lr_x0 = minX1;
        lr_n = J.paths >= 2 ? imax(0, maxX1 - minX1) : 0;
        rl_n = imax(0, W - minX1);
    }
    const int n_mine = dir == 0 ? lr_n : rl_n;
    const int Tn = imax(lr_n, rl_n);
    const int dx = dir == 0 ? 1 : -1;
    const int xs = dir == 0 ? lr_x0 : W - 1;   // step t of this chain is at x = xs + dx * t
    const int16_t* const Cg = J.C;
    int16_t* const Og = dir == 0 ? J.Vl : J.Vr;
    const int16_t* const Bg = J.base;
    const uint8_t* const Lg = J.left;
    const bool use_base = PYR && J.refine, adaptive = J.adaptive != 0;
    const int P2c = J.P2, minD = J.minD;
    const size_t prow = (size_t)yy * W;
    const size_t lrow = (size_t)yy * J.lstep;
    const long long dxD = (long long)dx * D;
    // issue cursor (step ti) and consume cursor (step t): voxel offset, pixel index, image index
    size_t oi = (prow + xs) * D + 2 * NW * k, pi = prow + xs, li = lrow + xs;
    size_t oc = oi, pc = pi, lc = li;
    int ti = 0;
    auto issue_next = [&](int slot) {
        if (ti < n_mine && PG_IN(oi, 2 * NW, (size_t)W * J.h * D, 5)) {
            cpw<NW>(ring + slot * 32 * RS, Cg + oi);
            if (use_base) cp4(bi + slot * 64, word_of(Bg + pi));
            if (adaptive) cp4(bi + slot * 64 + 32, word_of(Lg + li));
        }
        cp_commit();
        ++ti;
        oi += dxD;
        pi += dx;
        li += dx;
    };

    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    GChain<NW> s;
    gchain_init(s, minD);
#pragma unroll
    for (int j = 0; j < S - 1; ++j) issue_next(j);
    int img_prev = 0, slot = 0, islot = S - 1;
#pragma unroll 2
    for (int t = 0; t < Tn; ++t) {
        issue_next(islot);
        islot = islot + 1 == S ? 0 : islot + 1;
        cp_wait<S - 1>();
        const uint32_t* d = ring + slot * 32 * RS;
        const uint32_t* db = bi + slot * 64;
        slot = slot + 1 == S ? 0 : slot + 1;
        uint32_t cc[NW];
        ldw<NW>(d, cc);
        const int base = use_base ? (int)(int16_t)(db[0] >> ((pc & 1) * 16)) : minD;
        int p2 = P2c;
        if (adaptive) {
            const int img = (int)((db[32] >> byte_shift(Lg + lc)) & 255u);
            p2 = lut[abs(img - img_prev) & 255];
            img_prev = img;
        }
        if (PYR && !J.refine) {
            int lo, hi;
            label_range(J, xs + dx * t, minD, lo, hi);
            mask_labels<NW>(cc, lo, hi, k);
        }
        gstep<NW, T, PYR>(s, cc, base, p2, p12, chain + (G::NBUF == 2 ? (t & 1) * G::BUFW : 0), k);
        if (t < n_mine && row_ok && PG_IN(oc, 2 * NW, (size_t)W * J.h * D, 6))
            stw<NW>(reinterpret_cast<uint32_t*>(Og + oc), s.L);
        oc += dxD;
        pc += dx;
        lc += dx;
    }
    cp_wait<0>();
}

// ---------------------------------------------------------------------------
// Winner-take-all of the packed levels, one thread per pixel, from the
// path costs in V (T->B), Vl and Vr (kernel_WTA_Subpixel,
// src/sgm_kernels.cu:573-640; pyramid kernel_PyramidWTA,
// src/sgm_kernels.cu:1290-1370).  Keys (cost << 7 | label) order by cost,
// then label, so one min tree gives the minimum and its first label.
// Single-scale pixels outside [minD + D, w + min(minD, 0)) and the last
// column are written invalid (no path finishes them in the reference).
// ---------------------------------------------------------------------------
template <int D, bool PYR, int NJ>
__global__ void __launch_bounds__(256) k_wta(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    constexpr int DW = D / 2;
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x = blockIdx.x * 32 + (threadIdx.x & 31);
    const int y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= J.w || y >= J.h) return;
    const int W = J.w;
    const size_t p = (size_t)y * W + x;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    bool wta = true;
    if (!PYR) {
        // the reference defines the aggregated volume on [minX1, maxX1)
        // (on [minX1, w) with one path) and picks winners on [minX1, maxX1)
        // except the last column
        const int minX1 = imax(J.minD + D, 0), maxX1 = W + imin(J.minD, 0);
        const int accEnd = J.paths >= 2 ? maxX1 : W;
        wta = x >= minX1 && x < maxX1 && x != W - 1;
        if (!(x >= minX1 && x < accEnd)) {
            J.disp_raw[p] = inv;
            J.conf_raw[p] = 0.0f;
            return;
        }
    }
    // three-path totals (order-free: one cap, SHRT_MAX sentinel)
    uint32_t t[DW];
    auto load = [&](const int16_t* v, uint32_t (&o)[DW]) {
#pragma unroll
        for (int i = 0; i < DW / 4; ++i) {
            const uint4 q = __ldg(reinterpret_cast<const uint4*>(v + p * D) + i);
            o[4 * i] = q.x; o[4 * i + 1] = q.y; o[4 * i + 2] = q.z; o[4 * i + 3] = q.w;
        }
    };
    load(J.Vr, t);
    if (J.paths >= 2) {
        uint32_t u[DW];
        load(J.Vl, u);
#pragma unroll
        for (int i = 0; i < DW; ++i) t[i] = gcombine<PYR>(u[i], t[i]);
    }
    if (J.paths >= 3) {
        uint32_t u[DW];
        load(J.V, u);
#pragma unroll
        for (int i = 0; i < DW; ++i) t[i] = gcombine<PYR>(u[i], t[i]);
    }
    __shared__ uint32_t tsh[DW * 256];   // word i of thread j at i * 256 + j
#pragma unroll
    for (int i = 0; i < DW; ++i) tsh[i * 256 + threadIdx.x] = t[i];
    if (J.debug_acc) {
#pragma unroll
        for (int i = 0; i < DW / 4; ++i)
            reinterpret_cast<uint4*>(J.V + p * D)[i] = make_uint4(t[4 * i], t[4 * i + 1], t[4 * i + 2], t[4 * i + 3]);
    }
    if (!wta) {
        J.disp_raw[p] = inv;
        J.conf_raw[p] = 0.0f;
        return;
    }
    auto key = [&](int d) -> unsigned {
        const uint32_t w = t[d >> 1];
        return (((d & 1) ? (w >> 16) : (w & 0xffffu)) << 7) | (unsigned)d;
    };
    unsigned best = 0xffffffffu;
#pragma unroll
    for (int d = 0; d < D; d += 2) best = umin(best, umin(key(d), key(d + 1)));
    const int minCost = (int)(best >> 7), bestD = (int)(best & 127u);
    unsigned a = 0xffffffffu;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const bool near = (unsigned)(d - bestD + 1) <= 2u;
        a = umin(a, near ? 0xffffffffu : key(d));
    }
    const int alt = (int)(a >> 7);
    auto half = [&](int d) -> int {
        return (int)((tsh[(d >> 1) * 256 + threadIdx.x] >> ((d & 1) * 16)) & 0xffffu);
    };
    const int c0 = bestD > 0 ? half(bestD - 1) : 0;
    const int c2 = bestD + 1 < D ? half(bestD + 1) : 0;
    const int base = (PYR && J.refine) ? (int)J.base[p] : J.minD;
    wta_out<D, PYR>(J, y, x, base, minCost, bestD, alt, c0, minCost, c2);
}

// ---------------------------------------------------------------------------
// Top -> bottom with the winner-take-all folded in: 16-label pyramid levels
// with all three paths, one thread per column chain, run after the row
// pass.  Each step a chain reads, beside its pixel's costs, the pixel's
// L->R and R->L path costs through the same cp.async ring, adds its own
// T->B costs to them (the one-cap sum is order-free) and picks the winner
// exactly as k_wta does.  The T->B costs are neither written nor read
// again: 96 bytes per pixel in plus the outputs, against 64 for k_gtb and
// 96 for k_wta.  Three ring slots of 3 x 1 KB per warp keep 16 warps per
// SM resident, enough for the 1080p level of 32 pairs in one wave.
// ---------------------------------------------------------------------------
namespace pk {
constexpr int kStagesTbw = 3;
constexpr int kTbwMinWarpsPerSm = 9;

__host__ __device__ constexpr size_t tbw_smem()
{
    using G = Grp<8, 1>;
    return 256 * 4 + (size_t)4 * 4 * (G::BUFW + kStagesTbw * 3 * 256 + kStagesTbw * 64);
}
}  // namespace pk

template <int NJ>
__global__ void __launch_bounds__(128, 4) k_gtbw(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace pk;
    using G = Grp<8, 1>;
    constexpr int D = 16, S = kStagesTbw, kWarps = 4, SLOT = 3 * 256;   // words: costs, Vl, Vr of 32 lanes
    const LevelDesc& J = jobs.d[blockIdx.y];
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    uint32_t* cbuf = smem + 256;
    uint32_t* rbuf = cbuf + kWarps * G::BUFW;
    uint32_t* bibuf = rbuf + kWarps * S * SLOT;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = threadIdx.x; i < kWarps * G::BUFW; i += blockDim.x) cbuf[i] = kMax2;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = J.w, H = J.h;
    const int col0 = (blockIdx.x * kWarps + warp) * 32;
    if (col0 >= W) return;   // the whole warp is past the image
    const int col = col0 + lane;
    const bool col_ok = col < W;
    const int x = imin(col, W - 1);
    uint32_t* chain = cbuf + warp * G::BUFW + lane;
    uint32_t* ring = rbuf + warp * S * SLOT + lane * 8;
    uint32_t* bi = bibuf + warp * S * 64 + lane;   // [slot][base, image][lane]
    const int h0 = ring_half(0, lane), h1 = ring_half(1, lane);
    const uint32_t p12 = dup(imin(J.P1, 0x8000));
    int lo = 0, hi = D - 1;
    if (!J.refine) label_range(J, x, J.minD, lo, hi);
    const bool use_base = J.refine != 0, adaptive = J.adaptive != 0;
    const int16_t* const Cg = J.C;
    const int16_t* const Lp = J.Vl;
    const int16_t* const Rp = J.Vr;
    const int16_t* const Bg = J.base;
    const uint8_t* const Lg = J.left;
    const size_t vstep = (size_t)W * D, lstep = (size_t)J.lstep;
    size_t oi = (size_t)x * D, pi = x, li = x;   // issue cursor (row yi)
    size_t pc = pi, lc = li;                     // consume cursor (row y)
    int yi = 0;
    auto issue_next = [&](int slot) {
        if (yi < H && PG_IN(oi, D, (size_t)W * H * D, 7)) {
            uint32_t* d = ring + slot * SLOT;
            cp16(d + h0, Cg + oi);
            cp16(d + h1, Cg + oi + 8);
            cp16(d + 256 + h0, Lp + oi);
            cp16(d + 256 + h1, Lp + oi + 8);
            cp16(d + 512 + h0, Rp + oi);
            cp16(d + 512 + h1, Rp + oi + 8);
            if (use_base) cp4(bi + slot * 64, word_of(Bg + pi));
            if (adaptive) cp4(bi + slot * 64 + 32, word_of(Lg + li));
        }
        cp_commit();
        ++yi;
        oi += vstep;
        pi += W;
        li += lstep;
    };
    auto ld8 = [&](const uint32_t* d, uint32_t (&v)[8]) {
        const uint4 a = *reinterpret_cast<const uint4*>(d + h0);
        const uint4 b = *reinterpret_cast<const uint4*>(d + h1);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
        v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    };
    GChain<8> s;
    gchain_init(s, J.minD);
#pragma unroll
    for (int j = 0; j < S - 1; ++j) issue_next(j);
    int img_prev = 0, slot = 0, islot = S - 1;
    for (int y = 0; y < H; ++y) {
        issue_next(islot);
        islot = islot + 1 == S ? 0 : islot + 1;
        cp_wait<S - 1>();
        const uint32_t* d = ring + slot * SLOT;
        const uint32_t* db = bi + slot * 64;
        slot = slot + 1 == S ? 0 : slot + 1;
        uint32_t cc[8], t[8];
        ld8(d, cc);
        const int base = use_base ? (int)(int16_t)(db[0] >> ((pc & 1) * 16)) : J.minD;
        int p2 = J.P2;
        if (adaptive) {
            const int img = (int)((db[32] >> byte_shift(Lg + lc)) & 255u);
            p2 = lut[abs(img - img_prev) & 255];
            img_prev = img;
        }
        if (!J.refine) mask_labels<8>(cc, lo, hi, 0);
        gstep<8, 1, true>(s, cc, base, p2, p12, chain, 0);
        {
            uint32_t u[8];
            ld8(d + 512, t);   // R->L
            ld8(d + 256, u);   // L->R
#pragma unroll
            for (int i = 0; i < 8; ++i) t[i] = gtotal3(s.L[i], u[i], t[i]);
        }
        if (col_ok) {
            const size_t p = (size_t)y * W + x;
            if (J.debug_acc) {
                reinterpret_cast<uint4*>(J.V + p * D)[0] = make_uint4(t[0], t[1], t[2], t[3]);
                reinterpret_cast<uint4*>(J.V + p * D)[1] = make_uint4(t[4], t[5], t[6], t[7]);
            }
            int minCost, bestD, alt, c0, c2;
            wta16(t, minCost, bestD, alt, c0, c2);
            wta_out<D, true>(J, y, x, base, minCost, bestD, alt, c0, minCost, c2);
        }
        pc += W;
        lc += lstep;
    }
    cp_wait<0>();
}



template <int NW, int T, bool PYR, int NJ>
cudaError_t launch_paths_packed(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    using G = pk::Grp<NW, T>;
    cudaError_t err;
    bool any_tb = false;
    for (int i = 0; i < jobs.n; ++i) any_tb = any_tb || jobs.d[i].paths >= 3;
    // T->B and the horizontal paths only share the cost volume.  In the
    // spread shapes (launches with few rows, which leave most SMs idle) T->B
    // runs on a second stream beside the row pass, joined before the WTA;
    // launches that fill the GPU run them one after the other (side by side
    // they only contend).
    // 16-label pyramid levels, wide shape, three paths everywhere, and
    // columns for at least kTbwMinWarpsPerSm warps per SM: the row pass
    // first, then T->B with the winner-take-all (k_gtbw).  Its serial chain
    // step carries the winner's work, so with few warps per SM it loses to
    // k_gtb + k_wta: per launch, 16 pairs of 1080p, 1165 against 1031 us
    // at 6.3 warps per SM and 467 against 308 us at 3.2; at 12.6 warps per
    // SM (32 pairs) it is about 15 % faster.
    bool tbw = false;
    if constexpr (PYR && NW == 8 && T == 1) {
        long long cols = 0;
        tbw = tbw_mode() != 0;
        for (int i = 0; i < jobs.n; ++i) {
            tbw = tbw && jobs.d[i].paths >= 3;
            cols += jobs.d[i].w;
        }
        tbw = tbw && (tbw_mode() == 2 || cols >= 32LL * pk::kTbwMinWarpsPerSm * sm_count());
    }
    ForkStreams& fk = fork_streams(st);
    const bool fork = NW != 8 && any_tb && fk.aux != nullptr;
    cudaStream_t tbst = st;
    if (tbw) any_tb = false;
    if (fork) {
        if ((err = cudaEventRecord(fk.fork, st)) != cudaSuccess) return err;
        if ((err = cudaStreamWaitEvent(fk.aux, fk.fork, 0)) != cudaSuccess) return err;
        tbst = fk.aux;
    }
    if (any_tb) {
        Jobs<NJ> tbj = jobs;
        int n = 0;
        for (int i = 0; i < jobs.n; ++i)
            if (jobs.d[i].paths >= 3) tbj.d[n++] = jobs.d[i];
        tbj.n = n;
        constexpr size_t smem = pk::tb_smem<NW, T>();
        if ((err = cudaFuncSetAttribute(k_gtb<NW, T, PYR, NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem)) != cudaSuccess)
            return err;
        constexpr int kWarps = pk::warps_of<NW>();
        const int cols = kWarps * G::CPW;
        dim3 g((e.max_w + cols - 1) / cols, n);
        prof_begin(tbst);
        k_gtb<NW, T, PYR, NJ><<<g, kWarps * 32, smem, tbst>>>(tbj);
        count_launch();
        prof_end(PK_PATH_TB, jobs_vox(tbj) * 4 + jobs_px(tbj) * ((tbj.d[0].refine ? 2 : 0) + (tbj.d[0].adaptive ? 1 : 0)), tbst);
        if ((err = launched(tbst, "k_gtb")) != cudaSuccess) return err;
    }
    constexpr int kWarps = pk::warps_of<NW>();
    const int rows = kWarps * G::CPW / 2;
    dim3 g((e.max_h + rows - 1) / rows, jobs.n);
    // NW == 8 (many rows): warp-wide 128-byte chunk I/O; spread shapes: per-lane streams
    if constexpr (NW == 8) {
        constexpr size_t smem = pk::row_smem<NW, T>();
        if ((err = cudaFuncSetAttribute(k_grow<NW, T, PYR, NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem)) != cudaSuccess)
            return err;
        prof_begin(st);
        k_grow<NW, T, PYR, NJ><<<g, kWarps * 32, smem, st>>>(jobs);
    } else {
        constexpr size_t smem = pk::row_lane_smem<NW, T>();
        if ((err = cudaFuncSetAttribute(k_grow_lane<NW, T, PYR, NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem)) != cudaSuccess)
            return err;
        prof_begin(st);
        k_grow_lane<NW, T, PYR, NJ><<<g, kWarps * 32, smem, st>>>(jobs);
    }
    count_launch();
    if (prof_enabled()) {
        // algorithmic bytes: each horizontal path reads the cost volume and
        // writes its costs once
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double px = (double)d.w * d.h;
            by += px * d.D * 2 * (d.paths >= 2 ? 4 : 2) + px * 2 * ((d.refine ? 2 : 0) + (d.adaptive ? 1 : 0));
        }
        prof_end(PK_PATH_ROW, by, st);
    }
    if ((err = launched(st, NW == 8 ? "k_grow" : "k_grow_lane")) != cudaSuccess) return err;
    if (fork) {
        if ((err = cudaEventRecord(fk.join, fk.aux)) != cudaSuccess) return err;
        if ((err = cudaStreamWaitEvent(st, fk.join, 0)) != cudaSuccess) return err;
    }
    if constexpr (PYR && NW == 8 && T == 1) {
        if (tbw) {
            constexpr size_t smem = pk::tbw_smem();
            if ((err = cudaFuncSetAttribute(k_gtbw<NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
                cudaSuccess)
                return err;
            dim3 gt((e.max_w + 127) / 128, jobs.n);
            prof_begin(st);
            k_gtbw<NJ><<<gt, 128, smem, st>>>(jobs);
            count_launch();
            prof_end(PK_TBW, jobs_vox(jobs) * 6 + jobs_px(jobs) * ((jobs.d[0].refine ? 2 : 0) + (jobs.d[0].adaptive ? 1 : 0) + 10),
                     st);
            return launched(st, "k_gtbw");
        }
    }
    dim3 gw((e.max_w + 31) / 32, (e.max_h + 7) / 8, jobs.n);
    prof_begin(st);
    k_wta<G::D, PYR, NJ><<<gw, 256, 0, st>>>(jobs);
    count_launch();
    prof_end(PK_WTA, jobs_vox(jobs) * 2 * (jobs.d[0].paths >= 3 ? 3 : jobs.d[0].paths) + jobs_px(jobs) * (2 + 6 + 4), st);
    return launched(st, "k_wta");
}

}  // namespace pg
