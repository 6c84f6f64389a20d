// k_fused.cuh -- path aggregation of the 16-label pyramid levels in two
// passes over the cost volume instead of three path passes and a WTA pass:
//
//   k_tblr  T->B and L->R together, writing P = min(cap, TB + LR) into V
//   k_rlw   R->L, the three-path total P + RL and the winner-take-all
//           (uniqueness, edge and confidence rules, sub-pixel, disp2)
//
// Same recurrences as the reference's pyramid path kernels
// (src/sgm_kernels.cu:1191-1334) and winner rules
// (src/sgm_kernels.cu:1336-1478); the three path costs of a voxel are
// non-negative and clamped once at one cap with a SHRT_MAX sentinel, so
// min(cap, (TB + LR) + RL) is the reference's total in any order
// (src/sgm_kernels.cu:1326-1328, 1407-1411).
//
// k_tblr: a warp owns a band of 32 rows of one level and walks its columns
// on a skewed front: at step s lane t is at pixel (row t, column s - t).
// Its L->R chain is its own (registers and a private window buffer); the
// T->B chain of a column enters the band at lane 0, passes down one lane
// per step through shared memory (lane t hands its T->B costs of column x
// to lane t + 1, which reaches column x one step later), and leaves at lane
// 31 into a global edge buffer for the band below.  Both path costs of a
// voxel are in one thread at one step, so P is written once and nothing is
// re-read.  Bands are work units taken from a ticket counter in order
// (job-major, band-minor); a band only waits for the band above, whose
// ticket is smaller, so that band's warp is already running and every wait
// ends (the same argument as single-pass scans with dynamic tile ids).  The
// band above publishes how many columns of its edge it has written
// (st.release after the edge stores; the consumer reads the count with
// ld.acquire).  Each wait is bounded: past kWaitCycles the waiting warp
// records the stall in g_fused_stalls and goes on (its results are then
// wrong, never hung).
//
// Cost input of both kernels: 128-byte runs (4 pixels x 16 labels) copied
// with cp.async by the whole warp into per-lane ring slots, so every request
// is a whole line.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "k_paths_packed.cuh"
#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {

// Waits that ran out (see above), per translation unit that instantiates the
// fused kernels; read by pyrsgm_gb300_fused_stalls.
static __device__ unsigned g_fused_stalls;

namespace fz {

using pk::kMax2;
using pk::kOne2;

constexpr int kBand = 32;            // rows per unit: one warp, a lane per row
constexpr int kAhead = 8;            // steps of look-ahead of the copies
constexpr int kSlots = 3;            // cost-run slots per lane (kAhead < 4 * kSlots - 3)
constexpr int kRing = 16;            // per-lane base / image word ring (> kAhead, power of two)
constexpr int kEdgeChunk = 8;        // edge columns per publish and per load
constexpr int kEdgeWords = 12;       // words per edge entry: 8 path-cost words, mp | img << 16, base, 2 pad
constexpr int kPadW = 9;             // guard words before label 0 of a window (16 labels + 2 halves)
constexpr int kLenW = kPadW + 16 + 2;
constexpr int kBufW = kLenW * 32;    // one window buffer of a warp (word w of lane c at w * 32 + c)
constexpr long long kWaitCycles = 4000000000LL;   // about 2 s at 2 GHz

static_assert(kAhead < 4 * kSlots - 3, "a cost run slot is refilled only after its last read");
static_assert(kAhead <= kEdgeChunk, "an edge chunk loads one chunk ahead");

// Control words of a job, at the start of its (otherwise unused) Vl buffer:
// [0] ticket of a launch whose first job this is, [1] spare, [2 + b] columns
// of band b's bottom edge published; the edge entries follow at ctl_edge.
__host__ __device__ inline int n_bands(int h) { return (h + kBand - 1) / kBand; }
__host__ __device__ inline size_t ctl_edge_bytes(int h) { return ((size_t)4 * (2 + n_bands(h)) + 255) & ~(size_t)255; }
// Bytes of Vl the fused pass uses (edges of every band but the last).
__host__ __device__ inline size_t ctl_bytes(int w, int h)
{
    return ctl_edge_bytes(h) + (size_t)(n_bands(h) - 1) * w * kEdgeWords * 4;
}

template <int NJ>
struct Units {
    int start[NJ + 1];   // first unit of job j; start[n] = total
    int total;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// One step of a 16-label chain whose previous path costs sit in `buf`
// (word w at w * 32; guard words kMax2): the shifted window for this
// pixel's label base, then the recurrence (the same arithmetic as
// pk::gstep for one thread per chain, pyramid rules).
__device__ __forceinline__ void step_from(const uint32_t* buf, int mp, int delta, const uint32_t (&c)[8], int p2,
                                          uint32_t p12, uint32_t (&L)[8], int& mp_out)
{
    delta = iclamp(delta, -17, 17);
    const int i0 = 2 * kPadW + delta - 1;
    const uint32_t* wp = buf + (i0 >> 1) * 32;
    const uint32_t sh = (uint32_t)(i0 & 1) * 16;
    uint32_t w0[10];
#pragma unroll
    for (int j = 0; j < 10; ++j) w0[j] = wp[j * 32];
    uint32_t w[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) w[j] = __funnelshift_r(w0[j], w0[j + 1], sh);
    const int lj = imin(0x7fff, mp + p2);
    const uint32_t lj2 = pk::dup(lj), mp2 = pk::dup(mp);
    const uint32_t inc2 = mp < 0x7fff ? kOne2 : 0u;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const uint32_t n0 = __funnelshift_r(w[m], w[m + 1], 16);
        const uint32_t t = __viaddmin_u16x2(w[m], p12, lj2);
        const uint32_t best = __vimin3_u16x2(n0, t, w[m + 1] + p12);
        uint32_t v = __viaddmin_u16x2(c[m], best - mp2, kMax2);
        v |= pk::sign_mask2(best + inc2) & kMax2;
        L[m] = v;
    }
    uint32_t m2 = __vminu2(__vimin3_u16x2(L[0], L[1], L[2]), __vimin3_u16x2(L[3], L[4], L[5]));
    m2 = __vimin3_u16x2(m2, L[6], L[7]);
    mp_out = imin((int)(m2 & 0xffffu), (int)(m2 >> 16));
}

// Shared-memory column of 16-byte piece p (0..7) of lane t's run slot:
// conflict-free both for the skewed per-lane reads and for the cooperative
// copies (checked exhaustively for every step phase).
__device__ __forceinline__ int run_col(int p, int t) { return (p ^ ((t >> 2) & 1)) << 2; }

template <int NJ>
constexpr size_t tblr_smem()
{
    // lut, T->B windows x2, L->R window, meta x2, edge chunks x2, cost runs, base/image ring
    return 4 * (256 + 3 * kBufW + 2 * 32 * 2 + 2 * kEdgeChunk * kEdgeWords + 32 * kSlots * 32 + kRing * 64);
}

}  // namespace fz

template <int NJ>
__global__ void __launch_bounds__(32) k_fused_reset(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.x];
    unsigned* ctl = reinterpret_cast<unsigned*>(J.Vl);
    const int n = 2 + fz::n_bands(J.h);
    for (int i = threadIdx.x; i < n; i += blockDim.x) ctl[i] = 0u;
}

// ---------------------------------------------------------------------------
// T->B + L->R (see the file comment).  Persistent: each block (one warp)
// takes band units from the ticket counter until none is left.
// ---------------------------------------------------------------------------
template <int NJ>
__global__ void __launch_bounds__(32) k_tblr(const __grid_constant__ Jobs<NJ> jobs,
                                             const __grid_constant__ fz::Units<NJ> units)
{
    using namespace fz;
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    uint32_t* twin = smem + 256;                 // [2][kBufW]  T->B windows, written by the lane above
    uint32_t* lwin = twin + 2 * kBufW;           // [kBufW]     L->R windows
    uint32_t* meta = lwin + kBufW;               // [2][32][2]  producer (mp | img << 16, base)
    uint32_t* ebuf = meta + 2 * 64;              // [2][kEdgeChunk][kEdgeWords]
    uint32_t* cring = ebuf + 2 * kEdgeChunk * kEdgeWords;   // [32][kSlots][32]
    uint32_t* bring = cring + 32 * kSlots * 32;  // [kRing][2][32] base word, image word
    const int lane = threadIdx.x;
    for (int i = lane; i < 3 * kBufW; i += 32) twin[i] = kMax2;   // guards (never written again)
    unsigned* ticket = reinterpret_cast<unsigned*>(jobs.d[0].Vl);

    for (;;) {
        int u = 0;
        if (lane == 0) u = (int)atomicAdd(ticket, 1u);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= units.total) break;
        int j = 0;
        while (j + 1 < jobs.n && units.start[j + 1] <= u) ++j;
        const LevelDesc& J = jobs.d[j];
        const int b = u - units.start[j];
        const int W = J.w, H = J.h, nb = n_bands(H);
        const int y0 = b * kBand, y = y0 + lane, yy = imin(y, H - 1);
        const bool row_ok = y < H;
        const bool has_above = b > 0, has_below = b + 1 < nb;
        unsigned* ctl = reinterpret_cast<unsigned*>(J.Vl);
        uint32_t* E = reinterpret_cast<uint32_t*>(reinterpret_cast<unsigned char*>(J.Vl) + ctl_edge_bytes(H));
        const uint32_t* Ein = E + (size_t)(b - 1) * W * kEdgeWords;
        uint32_t* Eout = E + (size_t)b * W * kEdgeWords;
        const unsigned* flag_in = ctl + 2 + (b - 1);
        unsigned* flag_out = ctl + 2 + b;
        const bool use_base = J.refine != 0, adaptive = J.adaptive != 0;
        const int16_t* const Cg = J.C;
        int16_t* const Vg = J.V;
        const int16_t* const Bg = J.base;
        const uint8_t* const Lg = J.left;
        const int minD = J.minD, P2c = J.P2;
        const uint32_t p12 = pk::dup(imin(J.P1, 0x8000));
        __syncwarp();
        for (int i = lane; i < 256; i += 32) lut[i] = adaptive ? J.p2lut[i] : 0;
        __syncwarp();

        // edge of the band above: wait until `need` columns are published
        unsigned avail = 0;
        bool stalled = false;
        auto wait_cols = [&](int need) {
            if (!has_above || (int)avail >= need || stalled) return;
            unsigned v = 0;
            if (lane == 0) {
                v = ld_acquire(flag_in);
                if ((int)v < need) {
                    const long long t0 = clock64();
                    while ((int)(v = ld_acquire(flag_in)) < need) {
                        if (clock64() - t0 > kWaitCycles) {
                            atomicAdd(&g_fused_stalls, 1u);
                            v = 0x7fffffffu;
                            break;
                        }
                        __nanosleep(64);
                    }
                }
            }
            v = __shfl_sync(0xffffffffu, v, 0);
            __syncwarp();   // the edge loads of every lane come after lane 0's acquire
            if (v == 0x7fffffffu) stalled = true;
            avail = v;
        };
        // copy edge chunk k (columns 8k .. 8k+7) of the band above into ebuf[k & 1]
        auto load_edge = [&](int k) {
            if (!has_above) return;
            const int c0 = k * kEdgeChunk;
            if (c0 >= W) return;
            wait_cols(imin(c0 + kEdgeChunk, W));
            if (lane < kEdgeChunk * 3) {
                const int e = lane / 3, pc = lane - e * 3;
                if (c0 + e < W)
                    pk::cp16(ebuf + ((k & 1) * kEdgeChunk + e) * kEdgeWords + pc * 4,
                             Ein + (size_t)(c0 + e) * kEdgeWords + pc * 4);
            }
        };
        // copies issued at step s: the cost runs that lanes start at step
        // s + kAhead, this lane's base / image words for step s + kAhead,
        // and at every 8th step the next edge chunk
        auto issue = [&](int s) {
            const int sa = s + kAhead;
            {
                const int i = lane >> 2, q = lane & 3;
                const int t = (sa & 3) + 4 * i;          // target lane: its run starts at step sa
                const int xr = sa - t;                    // run start column (a multiple of 4)
                if (xr >= 0 && xr + q < W && y0 + t < H) {
                    const int slot = (xr >> 2) % kSlots;
                    uint32_t* dst = cring + (t * kSlots + slot) * 32;
                    const int16_t* src = Cg + ((size_t)(y0 + t) * W + xr + q) * 16;
                    pk::cp16(dst + run_col(2 * q, t), src);
                    pk::cp16(dst + run_col(2 * q + 1, t), src + 8);
                }
            }
            const int xb = sa - lane;
            if (xb >= 0 && xb < W) {
                uint32_t* bs = bring + (sa & (kRing - 1)) * 64 + lane;
                if (use_base) pk::cp4(bs, pk::word_of(Bg + (size_t)yy * W + xb));
                if (adaptive) pk::cp4(bs + 32, pk::word_of(Lg + (size_t)yy * J.lstep + xb));
            }
            if (s >= 0 && (s & (kEdgeChunk - 1)) == 0) load_edge((s >> 3) + 1);
            pk::cp_commit();
        };

        pk::GChain<8> lr;
        pk::gchain_init(lr, minD);
        int img_prev = 0;
        load_edge(0);
        for (int s = -kAhead; s < 0; ++s) issue(s);
        const int S = W + kBand - 1;
        for (int s = 0; s < S; ++s) {
            pk::cp_wait<kAhead - 1>();
            __syncwarp();
            issue(s);
            const int x = s - lane;
            const bool act = x >= 0 && x < W;
            const int xc = iclamp(x, 0, W - 1);
            // costs of (y, x)
            uint32_t cc[8];
            {
                const uint32_t* r = cring + (lane * kSlots + (xc >> 2) % kSlots) * 32;
                const int q = xc & 3;
                const uint4 a = *reinterpret_cast<const uint4*>(r + run_col(2 * q, lane));
                const uint4 c2 = *reinterpret_cast<const uint4*>(r + run_col(2 * q + 1, lane));
                cc[0] = a.x; cc[1] = a.y; cc[2] = a.z; cc[3] = a.w;
                cc[4] = c2.x; cc[5] = c2.y; cc[6] = c2.z; cc[7] = c2.w;
            }
            const uint32_t* bw = bring + (s & (kRing - 1)) * 64 + lane;
            const int base = use_base ? (int)(int16_t)(bw[0] >> (((uintptr_t)(Bg + (size_t)yy * W + xc) & 2) * 8))
                                      : minD;
            const int img = adaptive ? (int)((bw[32] >> pk::byte_shift(Lg + (size_t)yy * J.lstep + xc)) & 255u) : 0;
            if (!J.refine) {
                int lo, hi;
                label_range(J, xc, minD, lo, hi);
                pk::mask_labels<8>(cc, lo, hi, 0);
            }
            // T->B input: the band above's edge (lane 0) or the lane above
            uint32_t* tw = twin + (s & 1) * kBufW + lane;
            int mp_tb, base_tb, img_tb;
            if (lane == 0) {
                if (has_above) {
                    const uint32_t* e = ebuf + (((s >> 3) & 1) * kEdgeChunk + (s & 7)) * kEdgeWords;
#pragma unroll
                    for (int i = 0; i < 8; ++i) tw[(kPadW + i) * 32] = e[i];
                    mp_tb = (int)(e[8] & 0xffffu);
                    img_tb = (int)(e[8] >> 16);
                    base_tb = (int)(int16_t)e[9];
                } else {
#pragma unroll
                    for (int i = 0; i < 8; ++i) tw[(kPadW + i) * 32] = kMax2;
                    mp_tb = 0x7fff;
                    img_tb = 0;
                    base_tb = minD;
                }
            } else {
                const uint2 m = *reinterpret_cast<const uint2*>(meta + ((s & 1) * 32 + lane) * 2);
                mp_tb = (int)(m.x & 0xffffu);
                img_tb = (int)(m.x >> 16);
                base_tb = (int)(int16_t)m.y;
            }
            uint32_t Ltb[8];
            int mtb;
            step_from(tw, mp_tb, base - base_tb, cc, adaptive ? lut[abs(img - img_tb) & 255] : P2c, p12, Ltb, mtb);
            // L->R
            uint32_t* lw = lwin + lane;
#pragma unroll
            for (int i = 0; i < 8; ++i) lw[(kPadW + i) * 32] = lr.L[i];
            uint32_t Llr[8];
            int mlr;
            step_from(lw, lr.mp, base - lr.prevBase, cc, adaptive ? lut[abs(img - img_prev) & 255] : P2c, p12, Llr,
                      mlr);
            if (act) {
#pragma unroll
                for (int i = 0; i < 8; ++i) lr.L[i] = Llr[i];
                lr.mp = mlr;
                lr.prevBase = base;
                img_prev = img;
                if (row_ok) {
                    uint32_t P[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) P[i] = pk::gcombine<true>(Ltb[i], Llr[i]);
                    uint4* o = reinterpret_cast<uint4*>(Vg + ((size_t)y * W + x) * 16);
                    o[0] = make_uint4(P[0], P[1], P[2], P[3]);
                    o[1] = make_uint4(P[4], P[5], P[6], P[7]);
                }
            }
            // hand the T->B state of (y, x) on
            if (lane < 31) {
                uint32_t* nw = twin + ((s + 1) & 1) * kBufW + lane + 1;
#pragma unroll
                for (int i = 0; i < 8; ++i) nw[(kPadW + i) * 32] = Ltb[i];
                *reinterpret_cast<uint2*>(meta + (((s + 1) & 1) * 32 + lane + 1) * 2) =
                    make_uint2((uint32_t)mtb | ((uint32_t)img << 16), (uint32_t)(uint16_t)(int16_t)base);
            } else if (act && has_below) {
                uint4* e = reinterpret_cast<uint4*>(Eout + (size_t)x * kEdgeWords);
                e[0] = make_uint4(Ltb[0], Ltb[1], Ltb[2], Ltb[3]);
                e[1] = make_uint4(Ltb[4], Ltb[5], Ltb[6], Ltb[7]);
                e[2] = make_uint4((uint32_t)mtb | ((uint32_t)img << 16), (uint32_t)(uint16_t)(int16_t)base, 0u, 0u);
                if ((x & (kEdgeChunk - 1)) == kEdgeChunk - 1 || x == W - 1) st_release(flag_out, (unsigned)(x + 1));
            }
        }
        pk::cp_wait<0>();
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// R->L + winner-take-all.  A warp holds 32 rows (a lane per row, all at the
// same column); the costs and the partial sums P of a run of 4 columns come
// in as 128-byte runs copied by the whole warp (8 lanes per run).
// ---------------------------------------------------------------------------
namespace fz {
constexpr int kRlwSlots = 3;         // run slots per volume (two in flight)
constexpr int kRlwWarps = 2;
constexpr size_t rlw_smem()
{
    // lut, per warp: window, cost and P run slots, base / image words
    return 4 * (256 + (size_t)kRlwWarps * (kBufW + 2 * kRlwSlots * 32 * 32 + kRlwSlots * 4 * 64));
}
}  // namespace fz

template <int NJ>
__global__ void __launch_bounds__(fz::kRlwWarps * 32) k_rlw(const __grid_constant__ Jobs<NJ> jobs)
{
    using namespace fz;
    constexpr int CH = 4, SC = kRlwSlots, SLOTW = 32 * 32;
    const LevelDesc& J = jobs.d[blockIdx.y];
    extern __shared__ __align__(16) uint32_t smem[];
    int* lut = reinterpret_cast<int*>(smem);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* win = smem + 256 + warp * kBufW;
    uint32_t* ringC = smem + 256 + kRlwWarps * kBufW + warp * 2 * SC * SLOTW;
    uint32_t* ringP = ringC + SC * SLOTW;
    uint32_t* bi = smem + 256 + kRlwWarps * (kBufW + 2 * SC * SLOTW) + warp * SC * CH * 64 + lane;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) lut[i] = J.adaptive ? J.p2lut[i] : 0;
    for (int i = lane; i < kBufW; i += 32) win[i] = kMax2;
    __syncthreads();
    const int row0 = (blockIdx.x * kRlwWarps + warp) * 32;
    if (row0 >= J.h) return;
    const int W = J.w, H = J.h;
    const int y = row0 + lane;
    const bool row_ok = y < H;
    const int yy = imin(y, H - 1);
    const int16_t* const Cg = J.C;
    int16_t* const Vg = J.V;
    const int16_t* const Bg = J.base;
    const uint8_t* const Lg = J.left;
    const bool use_base = J.refine != 0, adaptive = J.adaptive != 0;
    const int P2c = J.P2, minD = J.minD;
    const size_t prow = (size_t)yy * W, lrow = (size_t)yy * J.lstep;
    // this lane's share of the run copies: piece pce of the runs of rows 4j + (lane >> 3)
    const int pce = lane & 7, cq = pce >> 1, coff = (pce & 1) * 8;
    auto piece_col = [](int chn, int p) { return chn * 32 + ((p ^ (chn & 7)) << 2); };
    const int NC = (W + CH - 1) / CH;
    int ci_issue = 0;
    auto issue_next = [&](int slot) {
        const int t = ci_issue * CH + (CH - 1 - cq);   // step of pixel cq of the run
        if (t < W) {
            const int x = W - 1 - t;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int r = 4 * j + (lane >> 3);
                if (row0 + r < H) {
                    const size_t src = ((size_t)(row0 + r) * W + x) * 16 + coff;
                    pk::cp16(ringC + slot * SLOTW + piece_col(r, pce), Cg + src);
                    pk::cp16(ringP + slot * SLOTW + piece_col(r, pce), Vg + src);
                }
            }
        }
        // label base and image bytes of this lane's row, one word per step
        uint32_t* bslot = bi + slot * CH * 64;
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            const int ts = ci_issue * CH + s;
            if (ts < W) {
                const int x = W - 1 - ts;
                if (use_base) pk::cp4(bslot + s * 32, pk::word_of(Bg + prow + x));
                if (adaptive) pk::cp4(bslot + (CH + s) * 32, pk::word_of(Lg + lrow + x));
            }
        }
        pk::cp_commit();
        ++ci_issue;
    };
    const uint32_t p12 = pk::dup(imin(J.P1, 0x8000));
    pk::GChain<8> st;
    pk::gchain_init(st, minD);
#pragma unroll
    for (int j = 0; j < SC - 1; ++j) issue_next(j);
    int img_prev = 0, slot = 0, islot = SC - 1;
    uint32_t* const chain = win + lane;
    for (int ci = 0; ci < NC; ++ci) {
        issue_next(islot);
        islot = islot + 1 == SC ? 0 : islot + 1;
        pk::cp_wait<SC - 1>();
        __syncwarp();
        const uint32_t* cin = ringC + slot * SLOTW;
        const uint32_t* pin = ringP + slot * SLOTW;
        const uint32_t* db = bi + slot * CH * 64;
#pragma unroll
        for (int s = 0; s < CH; ++s) {
            const int t = ci * CH + s;
            if (t >= W) break;   // the same for the whole warp
            const int q = CH - 1 - s;
            const int x = W - 1 - t;
            uint32_t cc[8], pp[8];
            {
                const uint4 a = *reinterpret_cast<const uint4*>(cin + piece_col(lane, 2 * q));
                const uint4 c2 = *reinterpret_cast<const uint4*>(cin + piece_col(lane, 2 * q + 1));
                cc[0] = a.x; cc[1] = a.y; cc[2] = a.z; cc[3] = a.w;
                cc[4] = c2.x; cc[5] = c2.y; cc[6] = c2.z; cc[7] = c2.w;
                const uint4 e = *reinterpret_cast<const uint4*>(pin + piece_col(lane, 2 * q));
                const uint4 f = *reinterpret_cast<const uint4*>(pin + piece_col(lane, 2 * q + 1));
                pp[0] = e.x; pp[1] = e.y; pp[2] = e.z; pp[3] = e.w;
                pp[4] = f.x; pp[5] = f.y; pp[6] = f.z; pp[7] = f.w;
            }
            const int base = use_base ? (int)(int16_t)(db[s * 32] >> (((prow + x) & 1) * 16)) : minD;
            int p2 = P2c;
            if (adaptive) {
                const int img = (int)((db[(CH + s) * 32] >> pk::byte_shift(Lg + lrow + x)) & 255u);
                p2 = lut[abs(img - img_prev) & 255];
                img_prev = img;
            }
            if (!J.refine) {
                int lo, hi;
                label_range(J, x, minD, lo, hi);
                pk::mask_labels<8>(cc, lo, hi, 0);
            }
#pragma unroll
            for (int i = 0; i < 8; ++i) chain[(kPadW + i) * 32] = st.L[i];
            uint32_t Lr[8];
            int mr;
            step_from(chain, st.mp, base - st.prevBase, cc, p2, p12, Lr, mr);
#pragma unroll
            for (int i = 0; i < 8; ++i) st.L[i] = Lr[i];
            st.mp = mr;
            st.prevBase = base;
            // three-path total and the winner
            uint32_t tot[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) tot[i] = pk::gcombine<true>(pp[i], Lr[i]);
            if (!row_ok) continue;
            if (J.debug_acc) {
                uint4* o = reinterpret_cast<uint4*>(Vg + ((size_t)y * W + x) * 16);
                o[0] = make_uint4(tot[0], tot[1], tot[2], tot[3]);
                o[1] = make_uint4(tot[4], tot[5], tot[6], tot[7]);
            }
            // keys (cost << 7 | label): the minimum and its first label
            auto key = [&](int d) -> unsigned {
                const uint32_t w = tot[d >> 1];
                return (((d & 1) ? (w >> 16) : (w & 0xffffu)) << 7) | (unsigned)d;
            };
            unsigned best = 0xffffffffu;
#pragma unroll
            for (int d = 0; d < 16; d += 2) best = umin(best, umin(key(d), key(d + 1)));
            const int minCost = (int)(best >> 7), bestD = (int)(best & 127u);
            unsigned a = 0xffffffffu;
#pragma unroll
            for (int d = 0; d < 16; ++d) {
                const bool near = (unsigned)(d - bestD + 1) <= 2u;
                a = umin(a, near ? 0xffffffffu : key(d));
            }
            int c0 = 0, c2 = 0;
#pragma unroll
            for (int d = 0; d < 16; ++d) {
                const int v = (int)(key(d) >> 7);
                c0 = d == bestD - 1 ? v : c0;
                c2 = d == bestD + 1 ? v : c2;
            }
            pk::wta_out<16, true>(J, y, x, base, minCost, bestD, (int)(a >> 7), c0, minCost, c2);
        }
        __syncwarp();
        slot = slot + 1 == SC ? 0 : slot + 1;
    }
    pk::cp_wait<0>();
}

// Whether a launch of 16-label pyramid jobs can take the fused passes: all
// three paths, and each job's Vl holds the control words and edges.
template <int NJ>
bool fused_applicable(const Jobs<NJ>& jobs)
{
    for (int i = 0; i < jobs.n; ++i) {
        const LevelDesc& d = jobs.d[i];
        if (d.D != 16 || !d.pyr || d.paths != 3 || !d.Vl) return false;
        if (fz::ctl_bytes(d.w, d.h) > (size_t)d.w * d.h * 16 * 2) return false;
    }
    return jobs.n > 0;
}


template <int NJ>
cudaError_t launch_paths_fused16(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    cudaError_t err;
    fz::Units<NJ> un;
    int total = 0;
    for (int i = 0; i < jobs.n; ++i) {
        un.start[i] = total;
        total += fz::n_bands(jobs.d[i].h);
    }
    for (int i = jobs.n; i <= NJ; ++i) un.start[i] = total;
    un.total = total;
    k_fused_reset<NJ><<<jobs.n, 32, 0, st>>>(jobs);
    count_launch();
    if ((err = launched(st, "k_fused_reset")) != cudaSuccess) return err;
    constexpr size_t smem = fz::tblr_smem<NJ>();
    if ((err = cudaFuncSetAttribute(k_tblr<NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return err;
    static int resident = 0;   // blocks per SM (one warp each) at this shared-memory size
    if (resident == 0) {
        int nb = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tblr<NJ>, 32, smem)) != cudaSuccess)
            return err;
        resident = nb > 0 ? nb : 1;
    }
    const int grid = std::min(total, resident * sm_count());
    prof_begin(st);
    k_tblr<NJ><<<grid, 32, smem, st>>>(jobs, un);
    count_launch();
    if (prof_enabled()) {
        // read the cost volume, write P; label base and image byte per pixel
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double px = (double)d.w * d.h;
            by += px * 16 * 2 * 2 + px * ((d.refine ? 2 : 0) + (d.adaptive ? 1 : 0));
        }
        prof_end(PK_TBLR, by, st);
    }
    if ((err = launched(st, "k_tblr")) != cudaSuccess) return err;
    constexpr size_t smem2 = fz::rlw_smem();
    if ((err = cudaFuncSetAttribute(k_rlw<NJ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2)) !=
        cudaSuccess)
        return err;
    const int rows = fz::kRlwWarps * 32;
    dim3 g((e.max_h + rows - 1) / rows, jobs.n);
    prof_begin(st);
    k_rlw<NJ><<<g, fz::kRlwWarps * 32, smem2, st>>>(jobs);
    count_launch();
    if (prof_enabled()) {
        // read the cost volume and P (and write P back as the total in debug mode); outputs and keys
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double px = (double)d.w * d.h;
            by += px * 16 * 2 * 2 + px * (2 + 4 + 4 + (d.refine ? 2 : 0) + (d.adaptive ? 1 : 0));
        }
        prof_end(PK_RLW, by, st);
    }
    return launched(st, "k_rlw");
}

}  // namespace pg
