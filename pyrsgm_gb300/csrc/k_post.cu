// k_post.cu -- 3x3 median, median-changed confidence reset and the output
// conversion of one level, fused into one pass; plus the path-kernel
// dispatch.  Reference: kernel_MedianFilter3x3, kernel_ClearChangedMedian-
// Confidence (src/sgm_kernels.cu:891-931), convertDispAndConfKernel
// (src/sgm_kernels.cu:1530-1551) and the output copies of
// pyrsgm_compute_level / pyrsgm_compute_single_scale
// (src/sgm_kernels.cu:1837-1858, 2053-2069).
#include "profiler.h"
#include "sgm_common.cuh"
#include "sgm_launch.h"

namespace pg {

template <bool PYR, int NJ>
cudaError_t launch_paths_mode(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st);

PathShape path_shape(int D)
{
    if (D <= 16) return {16, 1};
    if (D <= 32) return {32, 1};
    int k = 2;
    while (32 * k < D) k *= 2;
    return {32, k};
}

template <int NJ>
cudaError_t launch_paths(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    return jobs.d[0].pyr ? launch_paths_mode<true, NJ>(jobs, e, st) : launch_paths_mode<false, NJ>(jobs, e, st);
}

// 3x3 median of the interior by column sorts: each column of three is
// sorted once and shared by the three windows it belongs to; the median of
// the nine is the median of (largest column minimum, median of the column
// medians, smallest column maximum) -- the structure of the opt_med9
// network of Paeth / Devillard ("Fast median search: an ANSI C
// implementation").
__device__ __forceinline__ int med3(int a, int b, int c) { return imax(imin(a, b), imin(imax(a, b), c)); }

struct Col3 {
    int lo, mid, hi;
};
__device__ __forceinline__ Col3 sort3(int a, int b, int c)
{
    const int l = imin(a, b), h = imax(a, b);
    return {imin(l, c), imax(l, imin(h, c)), imax(h, c)};
}
__device__ __forceinline__ int median9(const Col3& a, const Col3& b, const Col3& c)
{
    return med3(imax(imax(a.lo, b.lo), c.lo), med3(a.mid, b.mid, c.mid), imin(imin(a.hi, b.hi), c.hi));
}

// One block: 128 x 16 pixels, a thread per 4 adjacent pixels of a row.  The
// (LR-checked) disparities of the tile and its one-pixel halo are computed
// once into shared memory; the median takes the in-image neighbours only
// (sorted, middle element) at the image border.
constexpr int kPoX = 128, kPoY = 16;

template <int NJ>
__global__ void __launch_bounds__(256) k_post(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x0 = blockIdx.x * kPoX, y0 = blockIdx.y * kPoY;
    if (x0 >= J.w || y0 >= J.h) return;
    const int W = J.w, H = J.h;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    // Levels aggregated by the packed kernels leave the LR check to this
    // pass (kernel_StrictPyramidLRCheck / kernel_PseudoLRCheck,
    // src/sgm_kernels.cu:825-889).
    const bool check = uses_packed(J.D) && (J.post & POST_LRCHECK);
    const bool med = (J.post & POST_MEDIAN) != 0;
    // The LR-checked disparities of the tile and its halo, staged in three
    // rounds so that each thread's loads are in flight together: its raw
    // disparities, then the disp2 keys they point at, then the decisions.
    __shared__ int16_t td[kPoY + 2][kPoX + 2];   // row r, column c: pixel (y0 - 1 + r, x0 - 1 + c)
    if (check || med) {
        constexpr int kN = (kPoY + 2) * (kPoX + 2), kPer = (kN + 255) / 256;
        int dv[kPer], xs[kPer], rowp[kPer];   // (a level has far fewer than 2^31 pixels)
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int i = threadIdx.x + 256 * k;
            const int r = i / (kPoX + 2), c = i - r * (kPoX + 2);
            const int yy = y0 - 1 + r, xx = x0 - 1 + c;
            const bool in = i < kN && yy >= 0 && yy < H && xx >= 0 && xx < W;
            rowp[k] = in ? yy * W : 0;
            xs[k] = in ? xx : -1;
            dv[k] = in ? (int)J.disp_raw[(size_t)rowp[k] + xx] : (int)inv;
        }
        if (check) {
            unsigned k0[kPer], k1[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                k0[k] = k1[k] = 0xffffffffu;
                if (xs[k] >= 0 && dv[k] != inv) {
                    const int r0 = xs[k] - (dv[k] >> 4), r1 = xs[k] - ((dv[k] + 15) >> 4);
                    if (r0 >= 0 && r0 < W) k0[k] = __ldg(J.keys + (size_t)rowp[k] + r0);
                    if (r1 >= 0 && r1 < W) k1[k] = __ldg(J.keys + (size_t)rowp[k] + r1);
                }
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const int d16 = dv[k], xx = xs[k];
                if (xx < 0 || d16 == inv) continue;
                const int d0 = d16 >> 4, d1 = (d16 + 15) >> 4;
                const int r0 = xx - d0, r1 = xx - d1;
                // disp2 of right pixel rx from its key (cost << 16 | 0xffff - x)
                auto disp2 = [&](unsigned key, int rx) -> int {
                    return key == 0xffffffffu ? (int)inv : (int)(0xffffu - (key & 0xffffu)) - rx;
                };
                const bool in0 = r0 >= 0 && r0 < W, in1 = r1 >= 0 && r1 < W;
                const int v0 = in0 ? disp2(k0[k], r0) : 0, v1 = in1 ? disp2(k1[k], r1) : 0;
                if (J.pyr) {
                    const bool ok = (in0 && v0 >= J.minD && abs(v0 - d0) <= J.maxdiff) ||
                                    (in1 && v1 >= J.minD && abs(v1 - d1) <= J.maxdiff);
                    dv[k] = ok ? d16 : (int)inv;
                } else {
                    const bool bad0 = in0 && v0 >= J.minD && abs(v0 - d0) > J.maxdiff;
                    const bool bad1 = in1 && v1 >= J.minD && abs(v1 - d1) > J.maxdiff;
                    dv[k] = (bad0 && bad1) ? (int)inv : d16;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int i = threadIdx.x + 256 * k;
            if (i < kN) (&td[0][0])[i] = (int16_t)dv[k];
        }
        __syncthreads();
    }
    const int tx = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int xb = x0 + 4 * tx;
    if (xb >= W) return;
    const int np = imin(4, W - xb);
#pragma unroll 1
    for (int ty = warp; ty < kPoY; ty += 8) {
        const int y = y0 + ty;
        if (y >= H) break;
        const size_t p = (size_t)y * W + xb;
        int dv[4], dn[4];
        float cf[4];
        int din[4];
        float cin[4];
        if (np == 4 && (p & 3) == 0) {   // 8- and 16-byte loads of the four pixels
            const uint2 a = *reinterpret_cast<const uint2*>(J.disp_raw + p);
            const float4 c = *reinterpret_cast<const float4*>(J.conf_raw + p);
            din[0] = (int)(int16_t)(a.x & 0xffffu);
            din[1] = (int)(int16_t)(a.x >> 16);
            din[2] = (int)(int16_t)(a.y & 0xffffu);
            din[3] = (int)(int16_t)(a.y >> 16);
            cin[0] = c.x; cin[1] = c.y; cin[2] = c.z; cin[3] = c.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int jj = imin(j, np - 1);
                din[j] = J.disp_raw[p + jj];
                cin[j] = J.conf_raw[p + jj];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int jj = imin(j, np - 1);
            const int d = (check || med) ? (int)td[ty + 1][4 * tx + 1 + jj] : din[j];
            dv[j] = d;
            cf[j] = (d != din[j]) ? 0.0f : cin[j];  // the check zeroes what it rejects
            dn[j] = d;
        }
        if (med) {
            const bool inner = xb > 0 && xb + 4 < W && y > 0 && y + 1 < H;
            if (inner) {
                Col3 c[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const int cc = 4 * tx + k;   // tile column of pixel column xb - 1 + k
                    c[k] = sort3(td[ty][cc], td[ty + 1][cc], td[ty + 2][cc]);
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) dn[j] = median9(c[j], c[j + 1], c[j + 2]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (j >= np) break;
                    const int x = xb + j;
                    int v[9];
                    int n = 0;
                    for (int dy = -1; dy <= 1; ++dy) {
                        if (y + dy < 0 || y + dy >= H) continue;
                        for (int dx = -1; dx <= 1; ++dx) {
                            if (x + dx < 0 || x + dx >= W) continue;
                            v[n++] = td[ty + 1 + dy][4 * tx + 1 + j + dx];
                        }
                    }
                    for (int i = 1; i < n; ++i) {
                        const int key = v[i];
                        int q = i - 1;
                        while (q >= 0 && v[q] > key) { v[q + 1] = v[q]; --q; }
                        v[q + 1] = key;
                    }
                    dn[j] = v[n / 2];
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                if (dn[j] != dv[j]) cf[j] = 0.0f;
            }
        }
        const bool vec = np == 4;
        if (J.out16 && PG_IN((size_t)y * J.out16_pitch + xb, np, (size_t)J.out16_pitch * H, 8)) {
            int16_t* o = J.out16 + (size_t)y * J.out16_pitch + xb;
            if (vec && ((reinterpret_cast<uintptr_t>(o) & 7) == 0)) {
                *reinterpret_cast<uint2*>(o) =
                    make_uint2((uint32_t)(uint16_t)dn[0] | ((uint32_t)(uint16_t)dn[1] << 16),
                               (uint32_t)(uint16_t)dn[2] | ((uint32_t)(uint16_t)dn[3] << 16));
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j < np) o[j] = (int16_t)dn[j];
            }
        }
        float f32[4], fc[4];
        const bool conv = J.out32 && J.outc;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float f = (int16_t)dn[j] / 16.0f;
            const bool ok = (int16_t)dn[j] != inv && f > 0.0f;
            f32[j] = ok ? f : 0.0f;
            fc[j] = conv ? (ok ? cf[j] : 0.0f) : cf[j];
        }
        auto store4 = [&](float* o, const float (&v)[4]) {
            if (vec && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
                *reinterpret_cast<float4*>(o) = make_float4(v[0], v[1], v[2], v[3]);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (j < np) o[j] = v[j];
            }
        };
        if (conv) {
            store4(J.out32 + (size_t)y * J.out32_pitch + xb, f32);
            store4(J.outc + (size_t)y * J.outc_pitch + xb, fc);
        } else if (J.outc && J.conf_only_copy) {
            store4(J.outc + (size_t)y * J.outc_pitch + xb, fc);
        }
    }
}

template <int NJ>
cudaError_t launch_post(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    dim3 g((e.max_w + kPoX - 1) / kPoX, (e.max_h + kPoY - 1) / kPoY, jobs.n);
    prof_begin(st);
    k_post<NJ><<<g, 256, 0, st>>>(jobs);
    count_launch();
    if (prof_enabled()) {
        double by = 0;
        for (int i = 0; i < jobs.n; ++i) {
            const LevelDesc& d = jobs.d[i];
            const double outb = (d.out16 ? 2 : 0) + (d.out32 ? 4 : 0) + (d.outc ? 4 : 0);
            by += (double)d.w * d.h * (6 + outb);
        }
        prof_end(PK_POST, by, st);
    }
    return launched(st, "k_post");
}

template cudaError_t launch_paths<1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_paths<kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_post<1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_post<kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);

}  // namespace pg
