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

// Median of nine by 19 compare-exchanges (the opt_med9 network of
// Paeth / Devillard, "Fast median search: an ANSI C implementation").
__device__ __forceinline__ void cx(int& a, int& b)
{
    const int t = imin(a, b);
    b = imax(a, b);
    a = t;
}
__device__ __forceinline__ int median9(int p0, int p1, int p2, int p3, int p4, int p5, int p6, int p7, int p8)
{
    cx(p1, p2); cx(p4, p5); cx(p7, p8); cx(p0, p1); cx(p3, p4); cx(p6, p7);
    cx(p1, p2); cx(p4, p5); cx(p7, p8); cx(p0, p3); cx(p5, p8); cx(p4, p7);
    cx(p3, p6); cx(p1, p4); cx(p2, p5); cx(p4, p7); cx(p4, p2); cx(p6, p4);
    cx(p4, p2);
    return p4;
}

// One block: 32 x 8 pixels.  The (LR-checked) disparities of the tile and
// its one-pixel halo are computed once into shared memory, then each thread
// takes the median of its 3x3 neighbourhood (the in-image neighbours only,
// sorted, middle element, at the image border).
template <int NJ>
__global__ void __launch_bounds__(256) k_post(const __grid_constant__ Jobs<NJ> jobs)
{
    const LevelDesc& J = jobs.d[blockIdx.z];
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
    if (x0 >= J.w || y0 >= J.h) return;
    const int W = J.w, H = J.h;
    const int16_t inv = (int16_t)((J.minD - 1) * 16);
    // Levels aggregated by the packed kernels leave the LR check to this
    // pass (kernel_StrictPyramidLRCheck / kernel_PseudoLRCheck,
    // src/sgm_kernels.cu:825-889).
    const bool check = uses_packed(J.D) && (J.post & POST_LRCHECK);
    const bool med = (J.post & POST_MEDIAN) != 0;
    auto disp_at = [&](int xx, int yy) -> int {
        const int d16 = J.disp_raw[(size_t)yy * W + xx];
        if (!check || d16 == inv) return d16;
        const unsigned* krow = J.keys + (size_t)yy * W;
        auto disp2 = [&](int rx) -> int {
            const unsigned k = krow[rx];
            return k == 0xffffffffu ? (int)inv : (int)(0xffffu - (k & 0xffffu)) - rx;
        };
        const int d0 = d16 >> 4, d1 = (d16 + 15) >> 4;
        const int r0 = xx - d0, r1 = xx - d1;
        if (J.pyr) {
            bool ok = false;
            if (r0 >= 0 && r0 < W) { const int v = disp2(r0); if (v >= J.minD && abs(v - d0) <= J.maxdiff) ok = true; }
            if (r1 >= 0 && r1 < W) { const int v = disp2(r1); if (v >= J.minD && abs(v - d1) <= J.maxdiff) ok = true; }
            return ok ? d16 : (int)inv;
        }
        bool bad0 = false, bad1 = false;
        if (r0 >= 0 && r0 < W) { const int v = disp2(r0); bad0 = v >= J.minD && abs(v - d0) > J.maxdiff; }
        if (r1 >= 0 && r1 < W) { const int v = disp2(r1); bad1 = v >= J.minD && abs(v - d1) > J.maxdiff; }
        return (bad0 && bad1) ? (int)inv : d16;
    };
    __shared__ int16_t td[10][34];
    if (check || med) {
        for (int i = threadIdx.x; i < 10 * 34; i += blockDim.x) {
            const int r = i / 34, c = i - r * 34;
            const int yy = y0 - 1 + r, xx = x0 - 1 + c;
            td[r][c] = (yy >= 0 && yy < H && xx >= 0 && xx < W) ? (int16_t)disp_at(xx, yy) : inv;
        }
        __syncthreads();
    }
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= W || y >= H) return;
    const size_t p = (size_t)y * W + x;
    const int d_in = J.disp_raw[p];
    int d = (check || med) ? (int)td[ty + 1][tx + 1] : d_in;
    float c = (d != d_in) ? 0.0f : J.conf_raw[p];  // the check zeroes what it rejects
    if (med) {
        int m;
        if (x > 0 && x + 1 < W && y > 0 && y + 1 < H) {
            m = median9(td[ty][tx], td[ty][tx + 1], td[ty][tx + 2], td[ty + 1][tx], td[ty + 1][tx + 1],
                        td[ty + 1][tx + 2], td[ty + 2][tx], td[ty + 2][tx + 1], td[ty + 2][tx + 2]);
        } else {
            int v[9];
            int n = 0;
            for (int dy = -1; dy <= 1; ++dy) {
                if (y + dy < 0 || y + dy >= H) continue;
                for (int dx = -1; dx <= 1; ++dx) {
                    if (x + dx < 0 || x + dx >= W) continue;
                    v[n++] = td[ty + 1 + dy][tx + 1 + dx];
                }
            }
            for (int i = 1; i < n; ++i) {
                const int key = v[i];
                int j = i - 1;
                while (j >= 0 && v[j] > key) { v[j + 1] = v[j]; --j; }
                v[j + 1] = key;
            }
            m = v[n / 2];
        }
        if (m != d) c = 0.0f;
        d = m;
    }
    if (J.out16) J.out16[(size_t)y * J.out16_pitch + x] = (int16_t)d;
    if (J.out32 && J.outc) {
        const float f = (int16_t)d / 16.0f;
        const bool ok = (int16_t)d != inv && f > 0.0f;
        J.out32[(size_t)y * J.out32_pitch + x] = ok ? f : 0.0f;
        J.outc[(size_t)y * J.outc_pitch + x] = ok ? c : 0.0f;
    } else if (J.outc && J.conf_only_copy) {
        J.outc[(size_t)y * J.outc_pitch + x] = c;
    }
}

template <int NJ>
cudaError_t launch_post(const Jobs<NJ>& jobs, const LevelExtent& e, cudaStream_t st)
{
    dim3 g((e.max_w + 31) / 32, (e.max_h + 7) / 8, jobs.n);
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
    return cudaGetLastError();
}

template cudaError_t launch_paths<1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_paths<kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_post<1>(const Jobs<1>&, const LevelExtent&, cudaStream_t);
template cudaError_t launch_post<kBatchJobs>(const Jobs<kBatchJobs>&, const LevelExtent&, cudaStream_t);

}  // namespace pg
