// speckle.cu -- opt-in speckle filter on an int16 disparity map, after the
// SGM path (no counterpart in the reference library; its benchmark turns
// OpenCV's filterSpeckles off, bench/pyrsgm_bench.cpp:312-323).  Semantics
// of cv::filterSpeckles: 4-neighbours belong to one region when neither
// holds new_val and their values differ by at most max_diff; every region
// of at most max_speckle_size pixels is set to new_val.
//
// GPU form: connected components by lock-free union-find (roots linked
// larger index -> smaller with atomicCAS): first inside each 32x8 tile in
// shared memory, each pixel linking its right and lower neighbour, which
// leaves every pixel pointing at its tile-local root; then across tile
// borders in global memory; then root sizes (atomicAdd, one per distinct
// root and warp) and one pass that clears small regions.  The partition into
// regions is unique, so the output is exactly that of a sequential flood
// fill.
#include <cuda_runtime.h>

#include <cstdint>

#include "pyrsgm/pyrsgm_gb300.h"
#include "sgm_launch.h"

namespace pg {
namespace {

// Root of x; path halving (each visited node is pointed at its grandparent,
// an ancestor, so concurrent halving keeps every pointer valid).  Parents
// only ever point to smaller indices, so the walk ends within x steps.
__device__ __forceinline__ int sp_find(int* lab, int x)
{
    for (;;) {
        const int p = *(volatile int*)&lab[x];
        if (p == x) return x;
        const int gp = *(volatile int*)&lab[p];
        if (gp != p) lab[x] = gp;
        x = p;
    }
}

// Link the sets of a and b.  Every failed CAS means another thread linked a
// root meanwhile (the number of roots only falls), so the loop is lock-free;
// the bound is a guard, not a wait.
__device__ __forceinline__ void sp_union(int* lab, int a, int b, int n)
{
    for (int it = 0; it <= n; ++it) {
        a = sp_find(lab, a);
        b = sp_find(lab, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        if (atomicCAS(&lab[a], a, b) == a) return;
    }
}

struct SpArgs {
    short* d;
    size_t pitch;   // elements
    int w, h;
    int new_val, max_size, max_diff;
    int* lab;
    int* size;
};

__device__ __forceinline__ short sp_at(const SpArgs& A, int x, int y) { return A.d[(size_t)y * A.pitch + x]; }

// Tile pass: components inside one 32x8 tile (shared-memory union-find),
// then every pixel's global label is its tile-local root's pixel index.
__global__ void __launch_bounds__(256) k_sp_tile(const SpArgs A)
{
    __shared__ int lab[256];
    __shared__ short val[256];
    const int t = threadIdx.x, tx = t & 31, ty = t >> 5;
    const int x = blockIdx.x * 32 + tx, y = blockIdx.y * 8 + ty;
    const bool in = x < A.w && y < A.h;
    const short v = in ? sp_at(A, x, y) : (short)A.new_val;
    val[t] = v;
    lab[t] = v != A.new_val ? t : -1;
    __syncthreads();
    if (v != A.new_val) {
        if (tx + 1 < 32) {
            const short u = val[t + 1];
            if (u != A.new_val && abs(u - v) <= A.max_diff) sp_union(lab, t, t + 1, 256);
        }
        if (ty + 1 < 8) {
            const short u = val[t + 32];
            if (u != A.new_val && abs(u - v) <= A.max_diff) sp_union(lab, t, t + 32, 256);
        }
    }
    __syncthreads();
    if (!in) return;
    const int p = y * A.w + x;
    A.size[p] = 0;
    if (v == A.new_val) {
        A.lab[p] = -1;
        return;
    }
    const int r = sp_find(lab, t);
    A.lab[p] = (blockIdx.y * 8 + (r >> 5)) * A.w + blockIdx.x * 32 + (r & 31);
}

// Border pass: links across the right and lower edges of the tiles.
__global__ void k_sp_link(const SpArgs A)
{
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= A.w || y >= A.h) return;
    const bool right = (x & 31) == 31 && x + 1 < A.w, down = (y & 7) == 7 && y + 1 < A.h;
    if (!right && !down) return;
    const int v = sp_at(A, x, y);
    if (v == A.new_val) return;
    const int p = y * A.w + x, n = A.w * A.h;
    if (right) {
        const int u = sp_at(A, x + 1, y);
        if (u != A.new_val && abs(u - v) <= A.max_diff) sp_union(A.lab, p, p + 1, n);
    }
    if (down) {
        const int u = sp_at(A, x, y + 1);
        if (u != A.new_val && abs(u - v) <= A.max_diff) sp_union(A.lab, p, p + A.w, n);
    }
}

__global__ void __launch_bounds__(256) k_sp_count(const SpArgs A)
{
    const int lane = threadIdx.x & 31;
    const int x = blockIdx.x * 32 + lane, y = blockIdx.y * 8 + (threadIdx.x >> 5);
    int r = -1 - lane;   // outside the image or new_val: a key no other lane has
    if (x < A.w && y < A.h) {
        const int p = y * A.w + x;
        if (A.lab[p] >= 0) {
            r = sp_find(A.lab, p);
            A.lab[p] = r;
        }
    }
    // one atomic per distinct root in the warp (a large region's pixels
    // would otherwise queue on a single counter); all 32 lanes take part
    const unsigned peers = __match_any_sync(0xffffffffu, r);
    if (r >= 0 && lane == __ffs(peers) - 1) atomicAdd(&A.size[r], __popc(peers));
}

__global__ void k_sp_apply(const SpArgs A)
{
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= A.w || y >= A.h) return;
    const int p = y * A.w + x;
    if (A.lab[p] < 0) return;
    // the root again: path halving by other threads of the count pass may
    // have pointed lab[p] at an ancestor after its own thread stored the root
    const int r = sp_find(A.lab, p);
    if (A.size[r] <= A.max_size) A.d[(size_t)y * A.pitch + x] = (short)A.new_val;
}

}  // namespace
}  // namespace pg

extern "C" int pyrsgm_gb300_filter_speckles(short* d_disp, size_t pitch_bytes, int width, int height, short new_val,
                                            int max_speckle_size, int max_diff, cudaStream_t stream)
{
    if (!d_disp || width <= 0 || height <= 0 || pitch_bytes % sizeof(short) != 0 ||
        pitch_bytes < (size_t)width * sizeof(short) || max_diff < 0 || (long long)width * height > 0x7fffffffLL)
        return -1;
    if (max_speckle_size <= 0) return 0;
    const size_t n = (size_t)width * height;
    void* scratch = nullptr;
    if (cudaMallocAsync(&scratch, n * 8, stream) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    pg::SpArgs A{d_disp, pitch_bytes / sizeof(short), width, height, new_val, max_speckle_size, max_diff,
                 static_cast<int*>(scratch), static_cast<int*>(scratch) + n};
    const dim3 g((width + 31) / 32, (height + 7) / 8);
    cudaError_t e;
    pg::k_sp_tile<<<g, 256, 0, stream>>>(A);
    if ((e = pg::launched(stream, "k_sp_tile")) == cudaSuccess) {
        pg::k_sp_link<<<g, 256, 0, stream>>>(A);
        e = pg::launched(stream, "k_sp_link");
    }
    if (e == cudaSuccess) {
        pg::k_sp_count<<<g, 256, 0, stream>>>(A);
        e = pg::launched(stream, "k_sp_count");
    }
    if (e == cudaSuccess) {
        pg::k_sp_apply<<<g, 256, 0, stream>>>(A);
        e = pg::launched(stream, "k_sp_apply");
    }
    pg::count_launches(4);
    cudaFreeAsync(scratch, stream);
    return e == cudaSuccess ? 0 : -1;
}
