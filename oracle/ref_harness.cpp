// ref_harness.cpp -- runs the reference's own CUDA kernels on the GPU.
//
// TEST INFRASTRUCTURE ONLY.  The reference's src/sgm_kernels.cu and
// src/pyrdown.cu are compiled unmodified into device fatbins under
// oracle/_ref/ (oracle/build_oracle.py, from the reference sources).  This file is
// not reference code: it loads those fatbins through the CUDA runtime's
// library API and replays the reference's host-side launch schedule
// (grid/block/shared-memory sizes and kernel order) so that the reference
// kernels can be run on the same GPU and inputs as the product library and
// their outputs -- including the internal cost and aggregation volumes --
// compared bit for bit.  Citations are reference file:line.
//
// Exported with a ref_ prefix so it can be loaded beside the product library.

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

enum KernelId {
    K_FillDisp, K_BTGradPrecompute, K_BTCost, K_CensusCompute, K_CensusCost,
    K_BoxFilterH, K_BoxFilterV, K_PathLR, K_PathTB, K_PathRL_WTA,
    K_PseudoLRCheck, K_StrictPyramidLRCheck, K_Median, K_ClearChangedConf,
    K_InitCoarseLabels, K_PrepareRefineLabels, K_BTWindowCostLocal, K_CensusCostLocal,
    K_PathLRPyramid, K_PathTBPyramid, K_PathRLPyramidWTA, K_Convert, K_PyrDown, K_COUNT
};

// Source-level kernel names in the reference (src/sgm_kernels.cu, src/pyrdown.cu).
const char* kNames[K_COUNT] = {
    "kernel_FillDisp", "kernel_BTGradPrecompute", "kernel_BTCost", "kernel_CensusCompute",
    "kernel_CensusCost", "kernel_BoxFilterH", "kernel_BoxFilterV", "kernel_SGM_PathLR",
    "kernel_SGM_PathTB", "kernel_SGM_PathRL_WTA", "kernel_PseudoLRCheck",
    "kernel_StrictPyramidLRCheck", "kernel_MedianFilter3x3", "kernel_ClearChangedMedianConfidence",
    "kernel_InitCoarseLabels", "kernel_PrepareRefineLabels", "kernel_BTWindowCostLocal",
    "kernel_CensusCostLocal", "kernel_SGM_PathLRPyramid", "kernel_SGM_PathTBPyramid",
    "kernel_SGM_PathRLPyramidWTA", "convertDispAndConfKernel", "pyrDownKernel"};

cudaKernel_t g_k[K_COUNT] = {};
bool g_ready = false;
char g_err[512] = "ref harness not initialised";

// Unqualified function name of an Itanium-mangled symbol: "_Z<len><id>..."
// or "_ZN<len><id>...<len><id>E..." (the last component); a name without
// the _Z prefix (C linkage) is returned as is.
std::string baseName(const char* m)
{
    if (std::strncmp(m, "_Z", 2) != 0) return m;
    const char* p = m + 2;
    const bool nested = *p == 'N';
    if (nested) ++p;
    std::string last;
    while (*p >= '0' && *p <= '9') {
        size_t len = 0;
        while (*p >= '0' && *p <= '9') len = len * 10 + (size_t)(*p++ - '0');
        if (std::strlen(p) < len) return "";
        last.assign(p, len);
        p += len;
        if (!nested) break;
    }
    return last;
}

bool nameMatches(const char* mangled, const char* name) { return baseName(mangled) == name; }

bool loadLibrary(const char* path)
{
    cudaLibrary_t lib;
    cudaError_t e = cudaLibraryLoadFromFile(&lib, path, nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) {
        std::snprintf(g_err, sizeof g_err, "cudaLibraryLoadFromFile(%s): %s", path, cudaGetErrorString(e));
        return false;
    }
    unsigned n = 0;
    if (cudaLibraryGetKernelCount(&n, lib) != cudaSuccess) return false;
    std::vector<cudaKernel_t> ks(n);
    if (cudaLibraryEnumerateKernels(ks.data(), n, lib) != cudaSuccess) return false;
    for (cudaKernel_t k : ks) {
        const char* nm = nullptr;
        if (cudaFuncGetName(&nm, reinterpret_cast<const void*>(k)) != cudaSuccess || !nm) continue;
        for (int i = 0; i < K_COUNT; ++i)
            if (!g_k[i] && nameMatches(nm, kNames[i])) g_k[i] = k;
    }
    return true;
}

struct Args {
    std::vector<std::vector<uint8_t>> store;
    std::vector<void*> ptrs;
    template <class T> Args& operator<<(T v)
    {
        store.emplace_back(sizeof(T));
        std::memcpy(store.back().data(), &v, sizeof(T));
        return *this;
    }
    void** finish()
    {
        ptrs.clear();
        for (auto& s : store) ptrs.push_back(s.data());
        return ptrs.data();
    }
};

cudaError_t launch(KernelId id, dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args& a)
{
    return cudaLaunchKernel(reinterpret_cast<const void*>(g_k[id]), grid, block, a.finish(), smem, st);
}

// PyrsgmWorkspace, src/sgm_kernels.cu:1486-1503
struct RefWorkspace {
    int width = 0, height = 0, disp = 0;
    unsigned char *d_grad1 = nullptr, *d_grad2 = nullptr;
    uint32_t *d_census1 = nullptr, *d_census2 = nullptr;
    short *d_cost_sad = nullptr, *d_cost_acc = nullptr;
    short *d_disp_raw = nullptr, *d_disp_med = nullptr, *d_disp2 = nullptr, *d_disp2_cost = nullptr;
    float* d_conf_raw = nullptr;
    short* d_base_disp = nullptr;
    unsigned char* d_valid_mask = nullptr;
};

void freeAll(RefWorkspace* ws)
{
    void* ps[] = {ws->d_grad1, ws->d_grad2, ws->d_census1, ws->d_census2, ws->d_cost_sad,
                  ws->d_cost_acc, ws->d_disp_raw, ws->d_disp_med, ws->d_disp2, ws->d_disp2_cost,
                  ws->d_conf_raw, ws->d_base_disp, ws->d_valid_mask};
    for (void* p : ps) if (p) cudaFree(p);
    int w = ws->width, h = ws->height, d = ws->disp;
    *ws = RefWorkspace();
    ws->width = w; ws->height = h; ws->disp = d;
}

// pyrsgm_ensure_workspace, src/sgm_kernels.cu:1553-1605
int ensureWs(RefWorkspace* ws, int w, int h, int D)
{
    if (!ws) return -1;
    if (ws->width == w && ws->height == h && ws->disp == D && ws->d_cost_sad) return 0;
    freeAll(ws);
    const size_t px = (size_t)w * h;
    bool ok = cudaMalloc(&ws->d_grad1, px) == cudaSuccess &&
              cudaMalloc(&ws->d_grad2, px) == cudaSuccess &&
              cudaMalloc(&ws->d_census1, px * 4) == cudaSuccess &&
              cudaMalloc(&ws->d_census2, px * 4) == cudaSuccess &&
              cudaMalloc(&ws->d_cost_sad, px * D * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_cost_acc, px * D * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_disp_raw, px * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_disp_med, px * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_disp2, px * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_disp2_cost, px * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_conf_raw, px * 4) == cudaSuccess &&
              cudaMalloc(&ws->d_base_disp, px * 2) == cudaSuccess &&
              cudaMalloc(&ws->d_valid_mask, px) == cudaSuccess;
    if (!ok) { freeAll(ws); return -1; }
    ws->width = w; ws->height = h; ws->disp = D;
    return 0;
}

constexpr int kBtTile = 64;       // BTCOST_TILE_X, src/sgm_kernels.cu:137
constexpr int kCensusThreads = 128; // CENSUS_THREADS, src/sgm_kernels.cu:36
constexpr int kCensusTile = 64;   // CENSUS_COST_TILE_X, src/sgm_kernels.cu:301

#define RCHK(expr) do { cudaError_t _e = (expr); if (_e != cudaSuccess) { \
    std::snprintf(g_err, sizeof g_err, "%s:%d %s", __FILE__, __LINE__, cudaGetErrorString(_e)); \
    return -1; } } while (0)

void sanitizeP2(int& adaptive, float& alpha, float& beta, float& lower, float& upper)
{
    if (alpha < 0.0f) alpha = 0.0f;
    beta = std::fmax(beta, 0.5f);
    upper = std::fmax(upper, 1.0f);
    lower = std::fmin(std::fmax(lower, 0.0f), upper);
    if (alpha <= 0.0f && lower >= 1.0f) adaptive = 0;
}

int postAndOutputs(RefWorkspace* ws, bool pyramid, int w, int h, int minD, int maxdiff, int post,
                   short* d_disp, size_t disp_step, float* d_df, size_t df_step, float* d_cf,
                   size_t cf_step, cudaStream_t st)
{
    dim3 b2(16, 16), g2((w + 15) / 16, (h + 15) / 16);
    if (post & 1) {
        Args a; a << ws->d_disp_raw << (const short*)ws->d_disp2 << ws->d_conf_raw << w << h << minD << maxdiff;
        RCHK(launch(pyramid ? K_StrictPyramidLRCheck : K_PseudoLRCheck, g2, b2, 0, st, a));
    }
    short* fin = ws->d_disp_raw;
    if (post & 2) {
        Args a; a << (const short*)ws->d_disp_raw << ws->d_disp_med << w << h;
        RCHK(launch(K_Median, g2, b2, 0, st, a));
        Args c; c << (const short*)ws->d_disp_raw << (const short*)ws->d_disp_med << ws->d_conf_raw << w << h;
        RCHK(launch(K_ClearChangedConf, g2, b2, 0, st, c));
        fin = ws->d_disp_med;
    }
    if (d_disp)
        RCHK(cudaMemcpy2DAsync(d_disp, disp_step, fin, (size_t)w * 2, (size_t)w * 2, h,
                               cudaMemcpyDeviceToDevice, st));
    const short inv = (short)((minD - 1) * 16);
    if (d_df && d_cf) {
        Args a;
        a << (const short*)fin << (const float*)ws->d_conf_raw << d_df << d_cf << w << h << w << w
          << (int)(df_step / sizeof(float)) << (int)(cf_step / sizeof(float)) << inv;
        RCHK(launch(K_Convert, g2, b2, 0, st, a));
    } else if (d_cf && pyramid) {
        RCHK(cudaMemcpy2DAsync(d_cf, cf_step, ws->d_conf_raw, (size_t)w * 4, (size_t)w * 4, h,
                               cudaMemcpyDeviceToDevice, st));
    }
    return 0;
}

int initLevelBuffers(RefWorkspace* ws, int w, int h, int minD, cudaStream_t st)
{
    dim3 b2(16, 16), g2((w + 15) / 16, (h + 15) / 16);
    const short inv = (short)((minD - 1) * 16);
    const short smax = SHRT_MAX;
    { Args a; a << ws->d_disp_raw << w << h << inv; RCHK(launch(K_FillDisp, g2, b2, 0, st, a)); }
    { Args a; a << ws->d_disp2 << w << h << inv; RCHK(launch(K_FillDisp, g2, b2, 0, st, a)); }
    { Args a; a << ws->d_disp2_cost << w << h << smax; RCHK(launch(K_FillDisp, g2, b2, 0, st, a)); }
    RCHK(cudaMemsetAsync(ws->d_conf_raw, 0, (size_t)w * h * sizeof(float), st));
    return 0;
}

} // namespace

extern "C" {

int ref_init(const char* sgm_fatbin, const char* pyrdown_fatbin)
{
    if (g_ready) return 0;
    if (!loadLibrary(sgm_fatbin) || !loadLibrary(pyrdown_fatbin)) return -1;
    for (int i = 0; i < K_COUNT; ++i) {
        if (!g_k[i]) {
            std::snprintf(g_err, sizeof g_err, "reference kernel %s not found in fatbins", kNames[i]);
            return -1;
        }
    }
    g_ready = true;
    return 0;
}

const char* ref_last_error(void) { return g_err; }

void* ref_create_workspace(void) { return new RefWorkspace(); }

void ref_destroy_workspace(void* p)
{
    auto* ws = static_cast<RefWorkspace*>(p);
    if (!ws) return;
    freeAll(ws);
    delete ws;
}

int ref_workspace_reserve(void* p, int w, int h, int D)
{
    if (!p || w <= 0 || h <= 0 || D <= 0 || D > 1024 || D % 16) return -1;
    return ensureWs(static_cast<RefWorkspace*>(p), w, h, D);
}

// Device pointers of the internal volumes ([y][x][d] int16) after a call.
void* ref_ws_cost(void* p) { return static_cast<RefWorkspace*>(p)->d_cost_sad; }
void* ref_ws_acc(void* p) { return static_cast<RefWorkspace*>(p)->d_cost_acc; }
void* ref_ws_base(void* p) { return static_cast<RefWorkspace*>(p)->d_base_disp; }
void* ref_ws_valid(void* p) { return static_cast<RefWorkspace*>(p)->d_valid_mask; }

int ref_copy_volumes(void* p, short* cost, short* acc, cudaStream_t st)
{
    auto* ws = static_cast<RefWorkspace*>(p);
    if (!ws || !ws->d_cost_sad) return -1;
    const size_t n = (size_t)ws->width * ws->height * ws->disp * sizeof(short);
    if (cost && cudaMemcpyAsync(cost, ws->d_cost_sad, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return -1;
    if (acc && cudaMemcpyAsync(acc, ws->d_cost_acc, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess) return -1;
    return 0;
}

// pyrsgm_pyrdown_u8, src/pyrdown.cu:56-74
int ref_pyrdown_u8(const unsigned char* src, size_t src_step, int sw, int sh,
                   unsigned char* dst, size_t dst_step, int dw, int dh, cudaStream_t st)
{
    if (!g_ready || !src || !dst || sw < 2 || sh < 2 || dw != (sw + 1) / 2 || dh != (sh + 1) / 2) return -1;
    dim3 b(32, 8), g((dw + 31) / 32, (dh + 7) / 8);
    Args a; a << src << (int)src_step << sw << sh << dst << (int)dst_step << dw << dh;
    RCHK(launch(K_PyrDown, g, b, 0, st, a));
    return 0;
}

// pyrsgm_compute_level, src/sgm_kernels.cu:1617-1862
int ref_compute_level(
    void* workspace, const unsigned char* L, const unsigned char* R,
    const short* pdisp, const float* pconf, short* d_disp, float* d_df, float* d_cf,
    size_t ls, size_t rs, size_t pds, size_t pcs, size_t ds, size_t dfs, size_t cfs,
    int w, int h, int pw, int ph, int D, int minD, int maxD, int bs, int P1, int P2,
    int uniq, int maxdiff, int pfc, int cost, int post, int paths, int refine, float minConf,
    int adaptive, float alpha, float beta, float lower, float upper, cudaStream_t st)
{
    if (!g_ready) return -1;
    if (!workspace || !L || !R || w <= 0 || h <= 0 || D <= 0 || D > 1024 || D % 16 || (refine && D > 256))
        return -1;
    if (refine && (!pdisp || !pconf || pw <= 0 || ph <= 0)) return -1;
    auto* ws = static_cast<RefWorkspace*>(workspace);
    maxD = std::min(maxD, w - 1);
    maxD = std::min(maxD, SHRT_MAX / 16);
    if (!refine) maxD = std::min(maxD, minD + D - 1);
    if (maxD < minD || ensureWs(ws, w, h, D) != 0) return -1;
    sanitizeP2(adaptive, alpha, beta, lower, upper);
    minConf = std::fmin(std::fmax(minConf, 0.0f), 1.0f);
    paths = std::clamp(paths, 1, 3);
    const size_t path_smem = 2 * D * sizeof(short) + ((D + 31) / 32) * sizeof(int);
    dim3 b2(16, 16), g2((w + 15) / 16, (h + 15) / 16);
    if (initLevelBuffers(ws, w, h, minD, st)) return -1;

    if (refine) {
        Args a; a << pdisp << pconf << pw << ph << (int)(pds / sizeof(short)) << (int)(pcs / sizeof(float))
                  << ws->d_base_disp << ws->d_valid_mask << w << h << minD << maxD << D << minConf;
        RCHK(launch(K_PrepareRefineLabels, g2, b2, 0, st, a));
    } else {
        Args a; a << ws->d_base_disp << ws->d_valid_mask << w << h << minD;
        RCHK(launch(K_InitCoarseLabels, g2, b2, 0, st, a));
    }

    if (cost == 1) {
        dim3 cg((w + kCensusThreads - 1) / kCensusThreads, h);
        size_t cs = (kCensusThreads + 4) * 5;
        { Args a; a << L << ws->d_census1 << w << h << (int)ls << w;
          RCHK(launch(K_CensusCompute, cg, kCensusThreads, cs, st, a)); }
        { Args a; a << R << ws->d_census2 << w << h << (int)rs << w;
          RCHK(launch(K_CensusCompute, cg, kCensusThreads, cs, st, a)); }
        if (refine) {
            dim3 lb(D, 4), lg((w + 3) / 4, h);
            Args a; a << (const uint32_t*)ws->d_census1 << (const uint32_t*)ws->d_census2
                      << (const short*)ws->d_base_disp << (const unsigned char*)ws->d_valid_mask
                      << ws->d_cost_sad << w << h << w << D << minD << maxD;
            RCHK(launch(K_CensusCostLocal, lg, lb, 0, st, a));
        } else {
            dim3 g((w + kCensusTile - 1) / kCensusTile, h);
            Args a; a << (const uint32_t*)ws->d_census1 << (const uint32_t*)ws->d_census2 << ws->d_cost_sad
                      << w << h << w << D << minD;
            RCHK(launch(K_CensusCost, g, D, 0, st, a));
        }
    } else {
        { Args a; a << L << ws->d_grad1 << w << h << (int)ls << w << pfc; RCHK(launch(K_BTGradPrecompute, g2, b2, 0, st, a)); }
        { Args a; a << R << ws->d_grad2 << w << h << (int)rs << w << pfc; RCHK(launch(K_BTGradPrecompute, g2, b2, 0, st, a)); }
        if (refine) {
            dim3 lb(D, 4), lg((w + 3) / 4, h);
            Args a; a << (const unsigned char*)ws->d_grad1 << (const unsigned char*)ws->d_grad2 << L << R
                      << (const short*)ws->d_base_disp << (const unsigned char*)ws->d_valid_mask << ws->d_cost_sad
                      << w << h << w << (int)ls << (int)rs << D << minD << maxD << bs;
            RCHK(launch(K_BTWindowCostLocal, lg, lb, 0, st, a));
        } else {
            dim3 g((w + kBtTile - 1) / kBtTile, h);
            size_t sm = 2 * (kBtTile + 2) + 2 * (kBtTile + D + 2);
            Args a; a << (const unsigned char*)ws->d_grad1 << (const unsigned char*)ws->d_grad2 << L << R
                      << ws->d_cost_sad << w << h << w << (int)ls << (int)rs << D << minD;
            RCHK(launch(K_BTCost, g, D, sm, st, a));
            Args bh; bh << (const short*)ws->d_cost_sad << ws->d_cost_acc << w << h << D << bs;
            RCHK(launch(K_BoxFilterH, h, D, 0, st, bh));
            Args bv; bv << (const short*)ws->d_cost_acc << ws->d_cost_sad << w << h << D << bs;
            RCHK(launch(K_BoxFilterV, w, D, 0, st, bv));
        }
    }

    auto pathArgs = [&](Args& a) {
        a << ws->d_cost_acc << (const short*)ws->d_cost_sad << (const short*)ws->d_base_disp
          << (const unsigned char*)ws->d_valid_mask << L << (int)ls << w << h << D << minD << maxD << P1 << P2;
    };
    if (paths >= 2) {
        Args a; pathArgs(a); a << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathLRPyramid, h, D, path_smem, st, a));
    }
    if (paths >= 3) {
        Args a; pathArgs(a); a << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathTBPyramid, w, D, path_smem, st, a));
    }
    {
        Args a;
        a << ws->d_cost_acc << (const short*)ws->d_cost_sad << (const short*)ws->d_base_disp
          << (const unsigned char*)ws->d_valid_mask << L << (int)ls
          << ws->d_disp_raw << ws->d_disp2 << ws->d_disp2_cost << ws->d_conf_raw
          << w << h << D << minD << maxD << P1 << P2 << uniq << minConf << (paths >= 2 ? 1 : 0)
          << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathRLPyramidWTA, h, D, path_smem, st, a));
    }
    return postAndOutputs(ws, true, w, h, minD, maxdiff, post, d_disp, ds, d_df, dfs, d_cf, cfs, st);
}

// pyrsgm_compute_single_scale, src/sgm_kernels.cu:1864-2076
int ref_compute_single_scale(
    void* workspace, const unsigned char* L, const unsigned char* R,
    short* d_disp, float* d_df, float* d_cf, size_t ls, size_t rs, size_t ds, size_t dfs, size_t cfs,
    int w, int h, int D, int minD, int bs, int P1, int P2, int uniq, int maxdiff, int pfc,
    int cost, int post, int paths, int adaptive, float alpha, float beta, float lower, float upper,
    cudaStream_t st)
{
    if (!g_ready) return -1;
    sanitizeP2(adaptive, alpha, beta, lower, upper);
    const int minX1 = std::max(minD + D, 0);
    const int maxX1 = w + std::min(minD, 0);
    paths = std::clamp(paths, 1, 3);
    auto* ws = static_cast<RefWorkspace*>(workspace);
    if (ensureWs(ws, w, h, D) != 0) return -1;
    const size_t path_smem = 2 * D * sizeof(short) + ((D + 31) / 32) * sizeof(int);
    dim3 b2(16, 16), g2((w + 15) / 16, (h + 15) / 16);
    if (initLevelBuffers(ws, w, h, minD, st)) return -1;
    if (cost == 1) {
        dim3 cg((w + kCensusThreads - 1) / kCensusThreads, h);
        size_t cs = (kCensusThreads + 4) * 5;
        { Args a; a << L << ws->d_census1 << w << h << (int)ls << w; RCHK(launch(K_CensusCompute, cg, kCensusThreads, cs, st, a)); }
        { Args a; a << R << ws->d_census2 << w << h << (int)rs << w; RCHK(launch(K_CensusCompute, cg, kCensusThreads, cs, st, a)); }
        dim3 g((w + kCensusTile - 1) / kCensusTile, h);
        Args a; a << (const uint32_t*)ws->d_census1 << (const uint32_t*)ws->d_census2 << ws->d_cost_sad
                  << w << h << w << D << minD;
        RCHK(launch(K_CensusCost, g, D, 0, st, a));
    } else {
        { Args a; a << L << ws->d_grad1 << w << h << (int)ls << w << pfc; RCHK(launch(K_BTGradPrecompute, g2, b2, 0, st, a)); }
        { Args a; a << R << ws->d_grad2 << w << h << (int)rs << w << pfc; RCHK(launch(K_BTGradPrecompute, g2, b2, 0, st, a)); }
        dim3 g((w + kBtTile - 1) / kBtTile, h);
        size_t sm = 2 * (kBtTile + 2) + 2 * (kBtTile + D + 2);
        Args a; a << (const unsigned char*)ws->d_grad1 << (const unsigned char*)ws->d_grad2 << L << R
                  << ws->d_cost_sad << w << h << w << (int)ls << (int)rs << D << minD;
        RCHK(launch(K_BTCost, g, D, sm, st, a));
        Args bh; bh << (const short*)ws->d_cost_sad << ws->d_cost_acc << w << h << D << bs;
        RCHK(launch(K_BoxFilterH, h, D, 0, st, bh));
        Args bv; bv << (const short*)ws->d_cost_acc << ws->d_cost_sad << w << h << D << bs;
        RCHK(launch(K_BoxFilterV, w, D, 0, st, bv));
    }
    if (paths >= 2) {
        Args a; a << ws->d_cost_acc << (const short*)ws->d_cost_sad << L << (int)ls << w << h << D
                  << minX1 << maxX1 << P1 << P2 << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathLR, h, D, path_smem, st, a));
    }
    if (paths >= 3) {
        Args a; a << ws->d_cost_acc << (const short*)ws->d_cost_sad << L << (int)ls << w << h << D
                  << P1 << P2 << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathTB, w, D, path_smem, st, a));
    }
    {
        Args a; a << ws->d_cost_acc << (const short*)ws->d_cost_sad << L << (int)ls
                  << ws->d_disp_raw << ws->d_disp2 << ws->d_disp2_cost << ws->d_conf_raw
                  << w << h << D << minD << P1 << P2 << uniq << maxdiff << (paths >= 2 ? 1 : 0)
                  << adaptive << alpha << beta << lower << upper;
        RCHK(launch(K_PathRL_WTA, h, D, path_smem, st, a));
    }
    return postAndOutputs(ws, false, w, h, minD, maxdiff, post, d_disp, ds, d_df, dfs, d_cf, cfs, st);
}

} // extern "C"
