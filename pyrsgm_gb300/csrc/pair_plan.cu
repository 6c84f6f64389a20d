// pair_plan.cu -- see pair_plan.h.
#include <algorithm>
#include <climits>
#include <cstring>
#include <stdexcept>
#include <string>

#include "pair_plan.h"
#include "pyrsgm/pyrsgm_c.h"

namespace pg {
namespace {

size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

struct Layout {
    std::array<size_t, PairPlan::kMaxLevels + 1> ws_off{}, img_off{}, out_off{};
    std::array<int, PairPlan::kMaxLevels + 1> p8{}, p16{}, p32{};
    size_t conf0_off = 0, lut_off = 0, total = 0;
};

Layout layoutOf(int w, int h, int levels, const std::array<pyrsgm::LevelInfo, 5>& info)
{
    Layout L;
    size_t total = 0;
    for (int level = 0; level <= levels; ++level) {
        const pyrsgm::LevelInfo& li = info[level];
        L.ws_off[level] = total;
        total += al256(Workspace::bytes_for(li.width, li.height, li.num_labels));
        if (level > 0) {
            L.p8[level] = (int)al256(li.width);
            L.p16[level] = (int)(al256((size_t)li.width * 2) / 2);
            L.p32[level] = (int)(al256((size_t)li.width * 4) / 4);
            L.img_off[level] = total;
            total += al256((size_t)L.p8[level] * li.height) * 2;
            L.out_off[level] = total;
            total += al256((size_t)L.p16[level] * 2 * li.height) + al256((size_t)L.p32[level] * 4 * li.height);
        }
    }
    L.conf0_off = total;
    total += al256((size_t)w * h * 4);
    L.lut_off = total;
    total += 1024;
    L.total = total;
    return L;
}

}  // namespace

size_t PairPlan::bytesFor(int w, int h, const pyrsgm::Params& v)
{
    std::array<pyrsgm::LevelInfo, 5> info{};
    pyrsgm::levelGeometry(w, h, v, info);
    return layoutOf(w, h, v.pyramid_levels, info).total;
}

PairPlan::PairPlan(int w, int h, const pyrsgm::Params& v, cudaStream_t st)
    : width(w), height(h), params(v), levels(v.pyramid_levels)
{
    pyrsgm::levelGeometry(w, h, params, info);
    const Layout L = layoutOf(w, h, levels, info);
    cudaError_t err = cudaMalloc(&arena, L.total);
    if (err != cudaSuccess) {
        arena = nullptr;
        cudaGetLastError();
        throw std::runtime_error(std::string("pyrsgm: arena allocation: ") + cudaGetErrorString(err));
    }
    arena_bytes = L.total;
    auto* base = static_cast<unsigned char*>(arena);
    for (int level = 0; level <= levels; ++level) {
        const pyrsgm::LevelInfo& li = info[level];
        ws[level].carve(base + L.ws_off[level], li.width, li.height, li.num_labels);
        ws[level].owned = false;
        ws[level].mem = base + L.ws_off[level];
        pitch8[level] = L.p8[level];
        pitch16[level] = L.p16[level];
        pitch32[level] = L.p32[level];
        if (level > 0) {
            pyrL[level] = base + L.img_off[level];
            pyrR[level] = pyrL[level] + al256((size_t)pitch8[level] * li.height);
            disp16[level] = reinterpret_cast<int16_t*>(base + L.out_off[level]);
            conf[level] =
                reinterpret_cast<float*>(base + L.out_off[level] + al256((size_t)pitch16[level] * 2 * li.height));
        }
    }
    conf0 = reinterpret_cast<float*>(base + L.conf0_off);
    lut = reinterpret_cast<int*>(base + L.lut_off);
    adaptive = params.adaptive_p2 ? 1 : 0;
    alpha = params.p2_alpha;
    beta = params.p2_beta;
    lower = params.p2_lower_mult;
    upper = params.p2_upper_mult;
    sanitize_p2(adaptive, alpha, beta, lower, upper);
    if (adaptive) {
        err = launch_p2_table(lut, params.p2, alpha, beta, lower, upper, st);
        if (err != cudaSuccess) {
            cudaFree(arena);
            arena = nullptr;
            throw std::runtime_error(std::string("pyrsgm: adaptive P2 table: ") + cudaGetErrorString(err));
        }
    }
}

PairPlan::~PairPlan()
{
    if (arena) cudaFree(arena);
}

int PairPlan::postFlags(int level) const
{
    // src/stereo_matcher.cpp:229-236
    if (level != 0) return PYRSGM_POST_LRCHECK;
    return (params.lr_check ? PYRSGM_POST_LRCHECK : 0) | (params.median_filter ? PYRSGM_POST_MEDIAN : 0);
}

LevelDesc PairPlan::levelDesc(int level) const
{
    const pyrsgm::LevelInfo& li = info[level];
    LevelDesc d;
    std::memset(&d, 0, sizeof d);
    d.w = li.width;
    d.h = li.height;
    d.D = li.num_labels;
    d.minD = params.min_disparity;
    d.pyr = levels > 0 ? 1 : 0;
    d.refine = li.refine ? 1 : 0;
    d.cost = params.cost_mode == pyrsgm::CostMode::Census ? COST_CENSUS : COST_BT;
    d.bs = li.block_size;
    d.pfc = params.pre_filter_cap;
    d.P1 = params.p1;
    d.P2 = params.p2;
    d.uniq = params.uniqueness_ratio;
    d.maxdiff = params.disp12_max_diff;
    d.post = postFlags(level);
    d.paths = params.num_paths;
    d.adaptive = adaptive;
    d.minConf = params.pyramid_min_confidence;
    d.conf_only_copy = d.pyr;
    if (d.pyr) {
        // pyrsgm_compute_level clamps, src/sgm_kernels.cu:1661-1665
        int maxD = std::min(li.max_disparity, li.width - 1);
        maxD = std::min(maxD, SHRT_MAX / 16);
        if (!li.refine) maxD = std::min(maxD, d.minD + d.D - 1);
        d.maxD = maxD;
    } else {
        d.maxD = d.minD + d.D - 1;
    }
    fill_workspace_ptrs(d, ws[level]);
    d.p2lut = lut;
    if (level > 0) {
        d.left = pyrL[level];
        d.right = pyrR[level];
        d.lstep = d.rstep = pitch8[level];
        d.out16 = disp16[level];
        d.out16_pitch = pitch16[level];
        d.outc = conf[level];
        d.outc_pitch = pitch32[level];
    }
    if (li.refine) {
        d.pdisp = disp16[level + 1];
        d.pconf = conf[level + 1];
        d.pd_pitch = pitch16[level + 1];
        d.pc_pitch = pitch32[level + 1];
        d.pw = info[level + 1].width;
        d.ph = info[level + 1].height;
    }
    return d;
}

LevelDesc PairPlan::level0(const uint8_t* L, size_t lp, const uint8_t* R, size_t rp, int16_t* d16, size_t d16p,
                           float* d32, size_t d32p, float* c, size_t cp) const
{
    LevelDesc d = levelDesc(0);
    float* oc = c;
    size_t ocp = cp;
    if (!oc && d32) {
        oc = conf0;
        ocp = (size_t)width * 4;
    }
    d.left = L;
    d.right = R;
    d.lstep = (int)lp;
    d.rstep = (int)rp;
    d.out16 = d16;
    d.out16_pitch = (int)(d16p / 2);
    d.out32 = d32;
    d.out32_pitch = (int)(d32p / 4);
    d.outc = oc;
    d.outc_pitch = (int)(ocp / 4);
    return d;
}

void PairPlan::pyrdownDescs(int level, const uint8_t* L, size_t lp, const uint8_t* R, size_t rp,
                            PyrDownDesc out[2]) const
{
    const pyrsgm::LevelInfo& par = info[level - 1];
    const pyrsgm::LevelInfo& li = info[level];
    const uint8_t* sl = level == 1 ? L : pyrL[level - 1];
    const uint8_t* sr = level == 1 ? R : pyrR[level - 1];
    const int sls = level == 1 ? (int)lp : pitch8[level - 1];
    const int srs = level == 1 ? (int)rp : pitch8[level - 1];
    out[0] = {sl, pyrL[level], sls, par.width, par.height, pitch8[level], li.width, li.height};
    out[1] = {sr, pyrR[level], srs, par.width, par.height, pitch8[level], li.width, li.height};
}

}  // namespace pg
