// check.h -- the checked build (compiled with -DPYRSGM_CHECKED into
// libpyrsgm_gb300_checked.so; the default library compiles all of this to
// nothing).
//
// Stand-in for a memory checker: at chosen global-memory accesses a kernel
// tests the element range against its buffer's extent; a failed test
// records the site number in a flag of its translation unit and skips the
// access (no trap: the context stays usable).  After every launch the host
// waits for the stream, reads and clears the flag and the launch error, and
// turns either into an error return with the kernel's name; the batch
// engine does not capture graphs in this build.  The first failure is kept
// for pyrsgm_gb300_check_report.
//
// Sites: 1, 2 k_gtb cost loads and path-cost stores; 3, 4 k_grow cost runs
// in and path-cost runs out; 5, 6 k_grow_lane loads and stores; 7 k_gtbw
// loads; 8 k_post disparity output; 9 k_features feature row; 10
// k_cost_census cost row; 11 k_cost_bt_tiled cost row; 12, 13 k_path_tb
// and k_path_row path-cost stores.
#pragma once

#include <cuda_runtime.h>

namespace pg {

// Host side (capi.cu): count a failure and keep the first message.
void check_record(const char* kernel, int site, cudaError_t err);
// 1 in the checked build.
constexpr bool kChecked =
#ifdef PYRSGM_CHECKED
    true;
#else
    false;
#endif

#ifdef PYRSGM_CHECKED
namespace {
__device__ unsigned g_check_site;   // first failing site of this translation unit (0: none)
}  // namespace

// Elements [i, i + len) inside [0, n)?  Records `site` and returns false if not.
__device__ __forceinline__ bool check_range(long long i, long long len, long long n, unsigned site)
{
    if (i >= 0 && i + len <= n) return true;
    atomicCAS(&g_check_site, 0u, site);
    return false;
}

// After a launch on `st`: the launch error; in the checked build also wait
// for the stream (unless a caller is capturing it) and report an execution
// error or a failed site.
static inline cudaError_t launched(cudaStream_t st, const char* kernel)
{
    cudaError_t err = cudaGetLastError();
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (err == cudaSuccess && cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
        return cudaSuccess;
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    unsigned site = 0;
    if (err == cudaSuccess) err = cudaMemcpyFromSymbol(&site, g_check_site, sizeof site);
    if (err == cudaSuccess && site != 0) {
        const unsigned zero = 0;
        cudaMemcpyToSymbol(g_check_site, &zero, sizeof zero);
        check_record(kernel, (int)site, cudaSuccess);
        return cudaErrorInvalidValue;
    }
    if (err != cudaSuccess) check_record(kernel, 0, err);
    return err;
}
#define PG_IN(i, len, n, site) ::pg::check_range((long long)(i), (long long)(len), (long long)(n), (site))
#else
static inline cudaError_t launched(cudaStream_t, const char*) { return cudaGetLastError(); }
#define PG_IN(i, len, n, site) true
#endif

}  // namespace pg
