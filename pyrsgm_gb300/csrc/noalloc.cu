// noalloc.cu -- pyrsgm_gb300_compute_level_noalloc: one pyramid level
// (same arguments and results as pyrsgm_compute_level, minus the workspace)
// for callers that must not allocate device memory.
//
// Who needs it.  Some hosts own every byte of device memory and do not let
// the code they load call cudaMalloc / cudaFree: robotics and automotive
// stacks that freeze the memory map after start-up, serving frameworks that
// hand plugins a fixed pool, and real-time loops where an allocation's
// implicit device synchronisation and unbounded latency would break the
// frame deadline.  pyrsgm_compute_level needs a workspace, and creating or
// growing one allocates; this entry point takes its scratch from a
// file-scope device array instead and calls no allocating routine.
//
// Limit.  The scratch is kNoAllocScratchBytes = 32 MiB.  Every GPU on which
// the library's device code is loaded holds it until the process exits.  A
// level fits when its workspace size -- pyrsgm_gb300_workspace_bytes(w, h, D),
// about w*h*(8*D + 44) bytes for 16/32/64 labels, w*h*(4*D + 44) otherwise --
// is at most 32 MiB, e.g. 480x360 with 16 labels or 256x192 with 64
// labels.  Larger levels are rejected with -1 and
// a message on stderr before any device work.
//
// Set-up.  Host code cannot use the array's name as a device address (on the
// host it is only a shadow symbol).  The first call on a device, with that
// device current, asks the runtime for the address once
// (cudaGetSymbolAddress) and caches it per device; make that first call
// before any stream capture.  The cached address belongs to the device's
// primary context: a call from another context on that device, or after
// cudaDeviceReset (which reloads the module, possibly elsewhere), would use
// a stale address, so neither is supported.
//
// Sharing.  All calls on a device use the same array and it keeps the last
// call's contents.  Nothing in it has to start at zero: every region a call
// reads is written earlier in that call.  Two calls whose GPU work overlaps
// (different streams, or host threads without ordering between them) race
// on the array; the caller must serialise them.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "pyrsgm/pyrsgm_c.h"
#include "pyrsgm/pyrsgm_gb300.h"
#include "sgm_launch.h"
#include "workspace.h"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (set up once per device).
int scratch_address(void** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return -1;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            std::fprintf(stderr, "pyrsgm-gb300 noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return -1;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return 0;
}

}  // namespace

extern "C" int pyrsgm_gb300_compute_level_noalloc(
    const unsigned char* d_left_gray, const unsigned char* d_right_gray, const short* d_parent_disp,
    const float* d_parent_conf, short* d_disp, float* d_disp_float, float* d_conf_float, size_t left_step_bytes,
    size_t right_step_bytes, size_t parent_disp_step_bytes, size_t parent_conf_step_bytes, size_t disp_step_bytes,
    size_t disp_float_step_bytes, size_t conf_float_step_bytes, int width, int height, int parent_width,
    int parent_height, int numDisparities, int minDisparity, int maxDisparity, int blockSize, int P1, int P2,
    int uniquenessRatio, int disp12MaxDiff, int preFilterCap, int costMode, int postFlags, int numPaths,
    int refineLevel, float minConfidence, int adaptiveP2, float p2Alpha, float p2Beta, float p2LowerMult,
    float p2UpperMult, cudaStream_t stream)
{
    // the argument rules of pyrsgm_compute_level
    if (!d_left_gray || !d_right_gray || width <= 0 || height <= 0 || numDisparities <= 0 ||
        numDisparities > 1024 || (numDisparities % 16) != 0 || (refineLevel && numDisparities > 256))
        return -1;
    if (refineLevel && (!d_parent_disp || !d_parent_conf || parent_width <= 0 || parent_height <= 0)) return -1;
    if (d_disp && (disp_step_bytes % sizeof(short)) != 0) return -1;
    const int D = numDisparities;
    const size_t need = pg::Workspace::bytes_for(width, height, D);
    if (need > kNoAllocScratchBytes) {
        std::fprintf(stderr,
                     "pyrsgm-gb300 noalloc: level %dx%d with %d labels needs %zu bytes of scratch; "
                     "the static scratch holds %zu\n",
                     width, height, D, need, kNoAllocScratchBytes);
        return -1;
    }
    maxDisparity = std::min(maxDisparity, width - 1);
    maxDisparity = std::min(maxDisparity, SHRT_MAX / 16);
    if (!refineLevel) maxDisparity = std::min(maxDisparity, minDisparity + D - 1);
    if (maxDisparity < minDisparity) return -1;

    void* scratch = nullptr;
    if (scratch_address(&scratch) != 0) return -1;
    pg::Workspace ws;
    ws.carve(static_cast<unsigned char*>(scratch), width, height, D);
    ws.mem = scratch;
    ws.owned = false;

    pg::sanitize_p2(adaptiveP2, p2Alpha, p2Beta, p2LowerMult, p2UpperMult);
    minConfidence = fminf(fmaxf(minConfidence, 0.0f), 1.0f);
    numPaths = std::min(std::max(numPaths, 1), 3);

    pg::LevelDesc d;
    std::memset(&d, 0, sizeof d);
    d.left = d_left_gray;
    d.right = d_right_gray;
    d.lstep = (int)left_step_bytes;
    d.rstep = (int)right_step_bytes;
    if (refineLevel) {
        d.pdisp = d_parent_disp;
        d.pconf = d_parent_conf;
        d.pd_pitch = (int)(parent_disp_step_bytes / sizeof(short));
        d.pc_pitch = (int)(parent_conf_step_bytes / sizeof(float));
        d.pw = parent_width;
        d.ph = parent_height;
    }
    d.out16 = d_disp;
    d.out16_pitch = (int)(disp_step_bytes / sizeof(short));
    d.out32 = d_disp_float;
    d.out32_pitch = (int)(disp_float_step_bytes / sizeof(float));
    d.outc = d_conf_float;
    d.outc_pitch = (int)(conf_float_step_bytes / sizeof(float));
    d.w = width;
    d.h = height;
    d.D = D;
    d.minD = minDisparity;
    d.maxD = maxDisparity;
    d.pyr = 1;
    d.refine = refineLevel ? 1 : 0;
    d.cost = costMode == PYRSGM_COST_CENSUS ? pg::COST_CENSUS : pg::COST_BT;
    d.bs = blockSize;
    d.pfc = preFilterCap;
    d.P1 = P1;
    d.P2 = P2;
    d.uniq = uniquenessRatio;
    d.maxdiff = disp12MaxDiff;
    d.post = postFlags;
    d.paths = numPaths;
    d.adaptive = adaptiveP2 ? 1 : 0;
    d.minConf = minConfidence;
    d.conf_only_copy = 1;
    pg::fill_workspace_ptrs(d, ws);
    return pg::run_level_single(d, stream, p2Alpha, p2Beta, p2LowerMult, p2UpperMult, "compute_level_noalloc");
}
