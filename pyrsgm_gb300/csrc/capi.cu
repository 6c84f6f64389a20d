// capi.cu -- the pyrsgm_c.h drop-in entry points (workspace, single-scale,
// per-level, pyrDown) on top of the batched launchers.
//
// Argument checks, parameter sanitising, clamps and error convention follow
// the reference host code (src/sgm_kernels.cu:1607-2076, src/pyrdown.cu:56-74).
// The kernel sequence differs: features -> (refine labels) -> cost ->
// (T->B) -> row pass (L->R + R->L + WTA + disp2 + LR check) -> median and
// outputs, 4-6 launches per level instead of ~17.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <utility>

#include "pyrsgm/pyrsgm_c.h"
#include "pyrsgm/pyrsgm_gb300.h"
#include "check.h"
#include "sgm_launch.h"
#include "workspace.h"
#include "trace.h"

namespace pg {

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// Failures seen by the checked build (check.h): how many, and the first.
static std::atomic<int> g_check_failures{0};
static std::mutex g_check_mu;
static char g_check_first[256] = {0};
void check_record(const char* kernel, int site, cudaError_t err)
{
    if (g_check_failures.fetch_add(1, std::memory_order_relaxed) == 0) {
        std::lock_guard<std::mutex> lk(g_check_mu);
        if (site != 0)
            std::snprintf(g_check_first, sizeof g_check_first, "%s: bounds check %d failed", kernel, site);
        else
            std::snprintf(g_check_first, sizeof g_check_first, "%s: %s", kernel, cudaGetErrorString(err));
    }
}

static std::atomic<int> g_packed_words{[] {
    const char* e = std::getenv("PYRSGM_GB300_PACKED_NW");
    return e ? std::atoi(e) : 0;
}()};
int packed_words_override() { return g_packed_words.load(std::memory_order_relaxed); }
static const int g_packed_wps = [] {
    const char* e = std::getenv("PYRSGM_GB300_PACKED_WPS");
    const int v = e ? std::atoi(e) : 0;
    return v > 0 && v <= 64 ? v : 1;
}();
int packed_min_warps_per_sm() { return g_packed_wps; }

static std::atomic<int> g_fused{[] {
    const char* e = std::getenv("PYRSGM_GB300_FUSED");
    return e && std::atoi(e) != 0 ? 1 : 0;
}()};
int fused_mode() { return g_fused.load(std::memory_order_relaxed); }

static std::atomic<int> g_tbw{[] {
    const char* e = std::getenv("PYRSGM_GB300_TBW");
    const int v = e ? std::atoi(e) : 1;
    return v >= 0 && v <= 2 ? v : 1;
}()};
int tbw_mode() { return g_tbw.load(std::memory_order_relaxed); }

static std::atomic<int> g_autotune{[] {
    const char* e = std::getenv("PYRSGM_GB300_AUTOTUNE");
    return e && std::atoi(e) != 0 ? 1 : 0;
}()};
static thread_local bool t_tuning = false;
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tune;
bool autotune_enabled() { return g_autotune.load(std::memory_order_relaxed) != 0; }
bool tuning_thread() { return t_tuning; }
TuningScope::TuningScope() : prev(t_tuning) { t_tuning = true; }
TuningScope::~TuningScope() { t_tuning = prev; }
bool tune_lookup(const TuneKey& k, TuneEntry& out)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(k);
    if (it == g_tune.end()) return false;
    out = it->second;
    return true;
}
void tune_store(const TuneKey& k, const TuneEntry& e)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[k] = e;
}

int sm_count()
{
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    std::atomic<int>& slot = cache[dev & 63];
    int n = slot.load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        slot.store(n, std::memory_order_relaxed);
    }
    return n;
}

ForkStreams& fork_streams(cudaStream_t st)
{
    // one auxiliary stream per (device, main stream) of this thread, so that
    // work forked from different main streams (server lanes) stays
    // independent; past 64 main streams they share one
    static thread_local std::map<std::pair<int, cudaStream_t>, ForkStreams> per;
    static thread_local ForkStreams none;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    auto key = std::make_pair(dev, per.size() < 64 ? st : nullptr);
    auto it = per.find(key);
    if (it != per.end()) return it->second;
    ForkStreams f;
    if (cudaStreamCreateWithFlags(&f.aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&f.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&f.join, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return none;
    }
    return per.emplace(key, f).first->second;
}

static size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t Workspace::bytes_for(int w, int h, int D)
{
    const size_t px = (size_t)w * h;
    return align256(px * 16) * 2 + align256(px * 2) + align256(px * D * 2) * (uses_packed(D) ? 4 : 2) +
           align256(px * 2) + align256(px * 4) * 2 + align256(256 * 4);
}

int Workspace::ensure(int w, int h, int D)
{
    if (w == width && h == height && D == disp && mem) return 0;
    release();
    const size_t n = bytes_for(w, h, D);
    if (cudaMalloc(&mem, n) != cudaSuccess) {
        mem = nullptr;
        cudaGetLastError();
        return -1;
    }
    carve(static_cast<unsigned char*>(mem), w, h, D);
    bytes = n;
    owned = true;
    return 0;
}

void Workspace::carve(unsigned char* p, int w, int h, int D)
{
    const size_t px = (size_t)w * h;
    featL = reinterpret_cast<uint4*>(p); p += align256(px * 16);
    featR = reinterpret_cast<uint4*>(p); p += align256(px * 16);
    base = reinterpret_cast<int16_t*>(p); p += align256(px * 2);
    C = reinterpret_cast<int16_t*>(p); p += align256(px * D * 2);
    V = reinterpret_cast<int16_t*>(p); p += align256(px * D * 2);
    Vl = Vr = nullptr;
    if (uses_packed(D)) {
        Vl = reinterpret_cast<int16_t*>(p); p += align256(px * D * 2);
        Vr = reinterpret_cast<int16_t*>(p); p += align256(px * D * 2);
    }
    disp_raw = reinterpret_cast<int16_t*>(p); p += align256(px * 2);
    conf_raw = reinterpret_cast<float*>(p); p += align256(px * 4);
    keys = reinterpret_cast<unsigned*>(p); p += align256(px * 4);
    lut = reinterpret_cast<int*>(p);
    width = w; height = h; disp = D;
}

void Workspace::release()
{
    if (mem && owned) cudaFree(mem);
    mem = nullptr;
    bytes = 0;
    width = height = disp = 0;
}

void sanitize_p2(int& adaptive, float& alpha, float& beta, float& lower, float& upper)
{
    // src/sgm_kernels.cu:1671-1676 and 1891-1895
    if (alpha < 0.0f) alpha = 0.0f;
    beta = fmaxf(beta, 0.5f);
    upper = fmaxf(upper, 1.0f);
    lower = fminf(fmaxf(lower, 0.0f), upper);
    if (alpha <= 0.0f && lower >= 1.0f) adaptive = 0;
}

void fill_workspace_ptrs(LevelDesc& d, const Workspace& ws)
{
    d.featL = ws.featL;
    d.featR = ws.featR;
    d.base = ws.base;
    d.C = ws.C;
    d.V = ws.V;
    d.Vl = ws.Vl;
    d.Vr = ws.Vr;
    d.disp_raw = ws.disp_raw;
    d.conf_raw = ws.conf_raw;
    d.keys = ws.keys;
    d.p2lut = ws.lut;
    d.debug_acc = ws.debug & PYRSGM_GB300_DEBUG_AGGREGATED;
}

int run_level_single(const LevelDesc& d, cudaStream_t st, float alpha, float beta, float lower, float upper,
                     const char* what)
{
    TraceRange tr("pyrsgm.%s (%dx%d, %d labels)", what, d.w, d.h, d.D);
    Jobs<1> j;
    j.d[0] = d;
    j.n = 1;
    const LevelExtent e = extent_of(j);
    cudaError_t err = cudaSuccess;
    if (d.adaptive) err = launch_p2_table(const_cast<int*>(d.p2lut), d.P2, alpha, beta, lower, upper, st);
    if (err == cudaSuccess) err = launch_prepare(j, e, st);
    if (err == cudaSuccess) err = launch_cost(j, e, st);
    if (err == cudaSuccess) err = launch_paths(j, e, st);
    if (err == cudaSuccess) err = launch_post(j, e, st);
    if (err != cudaSuccess) {
        std::fprintf(stderr, "pyrsgm-gb300 %s: %s\n", what, cudaGetErrorString(err));
        return -1;
    }
    return 0;
}

}  // namespace pg

using pg::LevelDesc;
using pg::Workspace;

extern "C" {

void* pyrsgm_create_workspace(void) { return new (std::nothrow) Workspace(); }

void pyrsgm_destroy_workspace(void* workspace)
{
    auto* ws = static_cast<Workspace*>(workspace);
    if (!ws) return;
    ws->release();
    delete ws;
}

int pyrsgm_workspace_reserve(void* workspace, int width, int height, int numDisparities)
{
    if (!workspace || width <= 0 || height <= 0 || numDisparities <= 0 || numDisparities > 1024 ||
        (numDisparities % 16) != 0)
        return -1;
    return static_cast<Workspace*>(workspace)->ensure(width, height, numDisparities);
}

int pyrsgm_pyrdown_u8(const unsigned char* d_src, size_t src_step_bytes, int src_width, int src_height,
                      unsigned char* d_dst, size_t dst_step_bytes, int dst_width, int dst_height,
                      cudaStream_t stream)
{
    if (!d_src || !d_dst || src_width < 2 || src_height < 2 || dst_width != (src_width + 1) / 2 ||
        dst_height != (src_height + 1) / 2)
        return -1;
    pg::PyrDownBatch<1> b;
    b.d[0] = {d_src, d_dst, (int)src_step_bytes, src_width, src_height, (int)dst_step_bytes, dst_width, dst_height};
    b.n = 1;
    return pg::launch_pyrdown(b, dst_width, dst_height, stream) == cudaSuccess ? 0 : -1;
}

int pyrsgm_compute_level(
    void* workspace, const unsigned char* d_left_gray, const unsigned char* d_right_gray,
    const short* d_parent_disp, const float* d_parent_conf, short* d_disp, float* d_disp_float,
    float* d_conf_float, size_t left_step_bytes, size_t right_step_bytes, size_t parent_disp_step_bytes,
    size_t parent_conf_step_bytes, size_t disp_step_bytes, size_t disp_float_step_bytes,
    size_t conf_float_step_bytes, int width, int height, int parent_width, int parent_height,
    int numDisparities, int minDisparity, int maxDisparity, int blockSize, int P1, int P2,
    int uniquenessRatio, int disp12MaxDiff, int preFilterCap, int costMode, int postFlags, int numPaths,
    int refineLevel, float minConfidence, int adaptiveP2, float p2Alpha, float p2Beta, float p2LowerMult,
    float p2UpperMult, cudaStream_t stream)
{
    // src/sgm_kernels.cu:1648-1678
    if (!workspace || !d_left_gray || !d_right_gray || width <= 0 || height <= 0 || numDisparities <= 0 ||
        numDisparities > 1024 || (numDisparities % 16) != 0 || (refineLevel && numDisparities > 256))
        return -1;
    if (refineLevel && (!d_parent_disp || !d_parent_conf || parent_width <= 0 || parent_height <= 0)) return -1;
    if (d_disp && (disp_step_bytes % sizeof(short)) != 0) return -1;
    auto* ws = static_cast<Workspace*>(workspace);
    const int D = numDisparities;
    maxDisparity = std::min(maxDisparity, width - 1);
    maxDisparity = std::min(maxDisparity, SHRT_MAX / 16);
    if (!refineLevel) maxDisparity = std::min(maxDisparity, minDisparity + D - 1);
    if (maxDisparity < minDisparity || ws->ensure(width, height, D) != 0) return -1;
    pg::sanitize_p2(adaptiveP2, p2Alpha, p2Beta, p2LowerMult, p2UpperMult);
    minConfidence = fminf(fmaxf(minConfidence, 0.0f), 1.0f);
    numPaths = std::min(std::max(numPaths, 1), 3);

    LevelDesc d;
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
    pg::fill_workspace_ptrs(d, *ws);
    return pg::run_level_single(d, stream, p2Alpha, p2Beta, p2LowerMult, p2UpperMult, "compute_level");
}

int pyrsgm_compute_single_scale(
    void* workspace, const unsigned char* d_left_gray, const unsigned char* d_right_gray, short* d_disp,
    float* d_disp_float, float* d_conf_float, size_t left_step_bytes, size_t right_step_bytes,
    size_t disp_step_bytes, size_t disp_float_step_bytes, size_t conf_float_step_bytes, int width, int height,
    int numDisparities, int minDisparity, int blockSize, int P1, int P2, int uniquenessRatio, int disp12MaxDiff,
    int preFilterCap, int costMode, int postFlags, int numPaths, int adaptiveP2, float p2Alpha, float p2Beta,
    float p2LowerMult, float p2UpperMult, cudaStream_t stream)
{
    // The reference performs no checks here beyond the allocation
    // (src/sgm_kernels.cu:1888-1907); a null image, an empty size or a label
    // count that is not a positive multiple of 16 (<= 1024) is rejected.
    if (!workspace || !d_left_gray || !d_right_gray || width <= 0 || height <= 0 || numDisparities <= 0 ||
        numDisparities > 1024 || (numDisparities % 16) != 0)
        return -1;
    if (d_disp && (disp_step_bytes % sizeof(short)) != 0) return -1;
    auto* ws = static_cast<Workspace*>(workspace);
    pg::sanitize_p2(adaptiveP2, p2Alpha, p2Beta, p2LowerMult, p2UpperMult);
    numPaths = std::min(std::max(numPaths, 1), 3);
    if (ws->ensure(width, height, numDisparities) != 0) {
        std::fprintf(stderr, "pyrsgm-gb300: workspace allocation failed\n");
        return -1;
    }
    LevelDesc d;
    std::memset(&d, 0, sizeof d);
    d.left = d_left_gray;
    d.right = d_right_gray;
    d.lstep = (int)left_step_bytes;
    d.rstep = (int)right_step_bytes;
    d.out16 = d_disp;
    d.out16_pitch = (int)(disp_step_bytes / sizeof(short));
    d.out32 = d_disp_float;
    d.out32_pitch = (int)(disp_float_step_bytes / sizeof(float));
    d.outc = d_conf_float;
    d.outc_pitch = (int)(conf_float_step_bytes / sizeof(float));
    d.w = width;
    d.h = height;
    d.D = numDisparities;
    d.minD = minDisparity;
    d.maxD = minDisparity + numDisparities - 1;
    d.pyr = 0;
    d.refine = 0;
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
    d.conf_only_copy = 0;  // single-scale writes confidence only together with disp_float
    pg::fill_workspace_ptrs(d, *ws);
    return pg::run_level_single(d, stream, p2Alpha, p2Beta, p2LowerMult, p2UpperMult, "compute_single_scale");
}

int pyrsgm_gb300_workspace_set_debug(void* workspace, int flags)
{
    if (!workspace) return -1;
    static_cast<Workspace*>(workspace)->debug = flags;
    return 0;
}

int pyrsgm_gb300_workspace_volumes(void* workspace, const short** cost, const short** aggregated, int* width,
                                   int* height, int* numDisparities)
{
    auto* ws = static_cast<Workspace*>(workspace);
    if (!ws || !ws->mem) return -1;
    if (cost) *cost = ws->C;
    if (aggregated) *aggregated = ws->V;
    if (width) *width = ws->width;
    if (height) *height = ws->height;
    if (numDisparities) *numDisparities = ws->disp;
    return 0;
}

int pyrsgm_gb300_workspace_copy_volumes(void* workspace, short* cost, short* aggregated, cudaStream_t stream)
{
    auto* ws = static_cast<Workspace*>(workspace);
    if (!ws || !ws->mem) return -1;
    const size_t n = (size_t)ws->width * ws->height * ws->disp * sizeof(short);
    if (cost && cudaMemcpyAsync(cost, ws->C, n, cudaMemcpyDeviceToDevice, stream) != cudaSuccess) return -1;
    if (aggregated && cudaMemcpyAsync(aggregated, ws->V, n, cudaMemcpyDeviceToDevice, stream) != cudaSuccess)
        return -1;
    return 0;
}

size_t pyrsgm_gb300_workspace_bytes(int width, int height, int numDisparities)
{
    if (width <= 0 || height <= 0 || numDisparities <= 0) return 0;
    return Workspace::bytes_for(width, height, numDisparities);
}

int pyrsgm_gb300_p2_table(int* d_table, int P2, float p2Alpha, float p2Beta, float p2LowerMult, float p2UpperMult,
                          cudaStream_t stream)
{
    if (!d_table) return -1;
    int adaptive = 1;
    pg::sanitize_p2(adaptive, p2Alpha, p2Beta, p2LowerMult, p2UpperMult);
    return pg::launch_p2_table(d_table, P2, p2Alpha, p2Beta, p2LowerMult, p2UpperMult, stream) == cudaSuccess ? 0
                                                                                                            : -1;
}

const char* pyrsgm_gb300_version(void) { return "0.1.0-gb300"; }

unsigned long long pyrsgm_gb300_launch_count(void) { return pg::g_launches.load(std::memory_order_relaxed); }

int pyrsgm_gb300_checked(void) { return pg::kChecked ? 1 : 0; }

int pyrsgm_gb300_check_report(char* first, size_t len)
{
    if (first && len > 0) {
        std::lock_guard<std::mutex> lk(pg::g_check_mu);
        std::snprintf(first, len, "%s", pg::g_check_first);
    }
    return pg::g_check_failures.load(std::memory_order_relaxed);
}

int pyrsgm_gb300_set_packed_words(int words)
{
    if (words != 0 && words != 2 && words != 4 && words != 8) return -1;
    return pg::g_packed_words.exchange(words, std::memory_order_relaxed);
}

int pyrsgm_gb300_set_fused(int on) { return pg::g_fused.exchange(on ? 1 : 0, std::memory_order_relaxed); }

int pyrsgm_gb300_set_tbw(int mode)
{
    if (mode < 0 || mode > 2) return -1;
    return pg::g_tbw.exchange(mode, std::memory_order_relaxed);
}

int pyrsgm_gb300_set_autotune(int on) { return pg::g_autotune.exchange(on ? 1 : 0, std::memory_order_relaxed); }

int pyrsgm_gb300_autotune_entries(pyrsgm_gb300_tune_entry* out, int capacity)
{
    std::lock_guard<std::mutex> lk(pg::g_tune_mu);
    int n = 0;
    for (const auto& kv : pg::g_tune) {
        if (out && n < capacity) {
            out[n].num_labels = kv.first.D;
            out[n].pyramid = kv.first.pyr;
            out[n].rows = kv.first.rows;
            out[n].width = kv.first.w;
            out[n].words = kv.second.nw;
            out[n].ms_wide = kv.second.ms_wide;
            out[n].ms_spread = kv.second.ms_spread;
        }
        ++n;
    }
    return n;
}

void pyrsgm_gb300_autotune_clear(void)
{
    std::lock_guard<std::mutex> lk(pg::g_tune_mu);
    pg::g_tune.clear();
}

}  // extern "C"
