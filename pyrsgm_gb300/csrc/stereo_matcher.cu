// stereo_matcher.cu -- pyrsgm::StereoMatcher (reference src/stereo_matcher.cpp)
// on one device arena.
//
// Same validation rules, level geometry, per-level post flags, scratch
// confidence and coarse-to-fine schedule as the reference
// (src/stereo_matcher.cpp:100-338).  Differences in how the work is laid out
// on the GPU: all buffers live in one allocation; the adaptive-P2 table is
// built once at construction (it depends on the parameters only); each
// pyramid level of both views is one pyrDown launch; each SGM level is the
// 4-5 fused launches of the level pipeline.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <string>

#include "pyrsgm/pyrsgm.h"
#include "pyrsgm/pyrsgm_c.h"
#include "pyrsgm/pyrsgm_gb300.h"
#include "pair_plan.h"
#include "trace.h"
#include "sgm_launch.h"
#include "workspace.h"

namespace pyrsgm {
namespace {

constexpr int kMaxLevels = 4;
constexpr int kRefineLabels = 16;
constexpr int kMaxCoarseLabels = 1024;

int align16(int v) { return std::max(16, ((v + 15) / 16) * 16); }

[[noreturn]] void throwCuda(const std::string& what, cudaError_t err)
{
    throw std::runtime_error("pyrsgm: " + what + ": " + cudaGetErrorString(err));
}

}  // namespace

// Level geometry of a validated parameter set, src/stereo_matcher.cpp:169-193.
void levelGeometry(int w, int h, const Params& params, std::array<LevelInfo, 5>& info)
{
    const int levels = params.pyramid_levels;
    int lw = w, lh = h;
    for (int level = 0; level <= levels; ++level) {
        if (level > 0) { lw = (lw + 1) / 2; lh = (lh + 1) / 2; }
        LevelInfo& li = info[level];
        li.level = level;
        li.width = lw;
        li.height = lh;
        if (levels == 0) {
            li.refine = false;
            li.num_labels = params.num_disparities;
            li.max_disparity = params.min_disparity + params.num_disparities - 1;
            li.block_size = params.block_size;
        } else {
            li.refine = level != levels;
            li.max_disparity = std::min(params.pyramid_max_disparity >> level, lw - 1);
            li.num_labels = li.refine ? kRefineLabels
                                      : align16(std::min(params.pyramid_coarse_disparities, li.max_disparity + 1));
            li.block_size = level >= 2 ? 3 : params.block_size;
        }
    }
}

Params validateParams(const Params& in)
{
    Params p = in;
    if (p.num_disparities <= 0 || p.num_disparities > kMaxCoarseLabels)
        throw std::invalid_argument("pyrsgm: num_disparities must be in (0, 1024]");
    p.num_disparities = align16(p.num_disparities);
    if (p.num_disparities > kMaxCoarseLabels)
        throw std::invalid_argument("pyrsgm: num_disparities must be <= 1024 after 16-alignment");
    if (p.block_size < 1) throw std::invalid_argument("pyrsgm: block_size must be >= 1");
    p.block_size = std::max(3, p.block_size | 1);
    if (p.p1 < 0 || p.p2 < p.p1) throw std::invalid_argument("pyrsgm: require 0 <= p1 <= p2");
    if (p.uniqueness_ratio < 0 || p.uniqueness_ratio >= 100)
        throw std::invalid_argument("pyrsgm: uniqueness_ratio must be in [0, 100)");
    if (p.pre_filter_cap <= 0) throw std::invalid_argument("pyrsgm: pre_filter_cap must be > 0");
    p.num_paths = std::clamp(p.num_paths, 1, 3);
    if (p.pyramid_levels < 0 || p.pyramid_levels > kMaxLevels)
        throw std::invalid_argument("pyrsgm: pyramid_levels must be in [0, 4]");
    if (p.pyramid_levels > 0) {
        if (p.min_disparity != 0) throw std::invalid_argument("pyrsgm: pyramid mode requires min_disparity = 0");
        if (p.disp12_max_diff < 0)
            throw std::invalid_argument("pyrsgm: pyramid mode requires disp12_max_diff >= 0");
        if (p.pyramid_coarse_disparities <= 0)
            throw std::invalid_argument("pyrsgm: pyramid_coarse_disparities must be > 0");
        p.pyramid_coarse_disparities = std::min(kMaxCoarseLabels, align16(p.pyramid_coarse_disparities));
        if (p.pyramid_max_disparity <= 0) p.pyramid_max_disparity = p.min_disparity + p.num_disparities - 1;
        if (p.pyramid_max_disparity < p.min_disparity)
            throw std::invalid_argument("pyrsgm: pyramid_max_disparity < min_disparity");
        p.pyramid_min_confidence = std::clamp(p.pyramid_min_confidence, 0.0f, 1.0f);
    }
    if (p.adaptive_p2 && p.p2_beta <= 0.0f) throw std::invalid_argument("pyrsgm: adaptive_p2 requires p2_beta > 0");
    return p;
}

struct StereoMatcher::Impl {
    pg::PairPlan plan;

    Impl(int w, int h, const Params& p) : plan(checkedSize(w, h), h, validateParams(p))
    {
        // the P2 table was enqueued on the legacy default stream; compute() may use any stream
        const cudaError_t err = cudaDeviceSynchronize();
        if (err != cudaSuccess) throwCuda("adaptive P2 table", err);
    }

    static int checkedSize(int w, int h)
    {
        if (w <= 0 || h <= 0) throw std::invalid_argument("pyrsgm: empty image size");
        return w;
    }

    void runLevel(const pg::LevelDesc& d, int level, cudaStream_t st)
    {
        pg::Jobs<1> j;
        j.d[0] = d;
        j.n = 1;
        const pg::LevelExtent e = pg::extent_of(j);
        cudaError_t err = pg::launch_prepare(j, e, st);
        if (err == cudaSuccess) err = pg::launch_cost(j, e, st);
        if (err == cudaSuccess) err = pg::launch_paths(j, e, st);
        if (err == cudaSuccess) err = pg::launch_post(j, e, st);
        if (err != cudaSuccess) {
            const LevelInfo& li = plan.info[level];
            std::ostringstream oss;
            oss << "pyramid level " << level << " (" << li.width << "x" << li.height << ", D=" << li.num_labels
                << ", refine=" << li.refine << ")";
            throwCuda(oss.str(), err);
        }
    }

    void compute(const uint8_t* L, size_t lp, const uint8_t* R, size_t rp, int16_t* d16, size_t d16p, float* d32,
                 size_t d32p, float* c, size_t cp, cudaStream_t st)
    {
        if (!L || !R) throw std::invalid_argument("pyrsgm: null input image");
        if (!d16 && !d32 && !c) return;
        if (d16 && (d16p % 2) != 0) throw std::invalid_argument("pyrsgm: disp16 pitch must be even");
        pg::TraceRange tr("pyrsgm.compute %dx%d L%d", plan.width, plan.height, plan.levels);
        // both views of a pyramid level in one launch
        for (int level = 1; level <= plan.levels; ++level) {
            pg::PyrDownBatch<2> b;
            b.n = 2;
            plan.pyrdownDescs(level, L, lp, R, rp, b.d);
            const cudaError_t err = pg::launch_pyrdown(b, plan.info[level].width, plan.info[level].height, st);
            if (err != cudaSuccess) throwCuda("pyrDown", err);
        }
        for (int level = plan.levels; level >= 0; --level) {
            const pg::LevelDesc d =
                level == 0 ? plan.level0(L, lp, R, rp, d16, d16p, d32, d32p, c, cp) : plan.levelDesc(level);
            pg::TraceRange tl("pyrsgm.level %d (%dx%d, %d labels)", level, d.w, d.h, d.D);
            runLevel(d, level, st);
        }
    }
};

StereoMatcher::StereoMatcher(int width, int height, const Params& params) : impl_(new Impl(width, height, params)) {}
StereoMatcher::~StereoMatcher() = default;
StereoMatcher::StereoMatcher(StereoMatcher&&) noexcept = default;
StereoMatcher& StereoMatcher::operator=(StereoMatcher&&) noexcept = default;

void StereoMatcher::compute(const uint8_t* d_left, size_t left_pitch, const uint8_t* d_right, size_t right_pitch,
                            int16_t* d_disp16, size_t disp16_pitch, float* d_disp32, size_t disp32_pitch,
                            float* d_conf, size_t conf_pitch, cudaStream_t stream)
{
    impl_->compute(d_left, left_pitch, d_right, right_pitch, d_disp16, disp16_pitch, d_disp32, disp32_pitch, d_conf,
                   conf_pitch, stream);
}

int StereoMatcher::width() const { return impl_->plan.width; }
int StereoMatcher::height() const { return impl_->plan.height; }
const Params& StereoMatcher::params() const { return impl_->plan.params; }
int StereoMatcher::numLevels() const { return impl_->plan.levels + 1; }
LevelInfo StereoMatcher::levelInfo(int level) const
{
    if (level < 0 || level > impl_->plan.levels) throw std::out_of_range("pyrsgm: level");
    return impl_->plan.info[level];
}
size_t StereoMatcher::deviceMemoryBytes() const { return impl_->plan.arena_bytes; }

const char* version() { return "0.1.0"; }

}  // namespace pyrsgm

// ---------------------------------------------------------------------------
// C surface over the C++ API (pyrsgm_gb300.h)
// ---------------------------------------------------------------------------
namespace {

pyrsgm::Params toParams(const pyrsgm_gb300_params& c)
{
    pyrsgm::Params p;
    p.num_disparities = c.num_disparities;
    p.min_disparity = c.min_disparity;
    p.block_size = c.block_size;
    p.cost_mode = c.cost_mode == PYRSGM_COST_CENSUS ? pyrsgm::CostMode::Census : pyrsgm::CostMode::BirchfieldTomasi;
    p.p1 = c.p1;
    p.p2 = c.p2;
    p.uniqueness_ratio = c.uniqueness_ratio;
    p.disp12_max_diff = c.disp12_max_diff;
    p.lr_check = c.lr_check != 0;
    p.median_filter = c.median_filter != 0;
    p.num_paths = c.num_paths;
    p.pre_filter_cap = c.pre_filter_cap;
    p.pyramid_levels = c.pyramid_levels;
    p.pyramid_coarse_disparities = c.pyramid_coarse_disparities;
    p.pyramid_max_disparity = c.pyramid_max_disparity;
    p.pyramid_min_confidence = c.pyramid_min_confidence;
    p.adaptive_p2 = c.adaptive_p2 != 0;
    p.p2_alpha = c.p2_alpha;
    p.p2_beta = c.p2_beta;
    p.p2_lower_mult = c.p2_lower_mult;
    p.p2_upper_mult = c.p2_upper_mult;
    return p;
}

pyrsgm_gb300_params fromParams(const pyrsgm::Params& p)
{
    pyrsgm_gb300_params c;
    c.num_disparities = p.num_disparities;
    c.min_disparity = p.min_disparity;
    c.block_size = p.block_size;
    c.cost_mode = p.cost_mode == pyrsgm::CostMode::Census ? PYRSGM_COST_CENSUS : PYRSGM_COST_BT;
    c.p1 = p.p1;
    c.p2 = p.p2;
    c.uniqueness_ratio = p.uniqueness_ratio;
    c.disp12_max_diff = p.disp12_max_diff;
    c.lr_check = p.lr_check;
    c.median_filter = p.median_filter;
    c.num_paths = p.num_paths;
    c.pre_filter_cap = p.pre_filter_cap;
    c.pyramid_levels = p.pyramid_levels;
    c.pyramid_coarse_disparities = p.pyramid_coarse_disparities;
    c.pyramid_max_disparity = p.pyramid_max_disparity;
    c.pyramid_min_confidence = p.pyramid_min_confidence;
    c.adaptive_p2 = p.adaptive_p2;
    c.p2_alpha = p.p2_alpha;
    c.p2_beta = p.p2_beta;
    c.p2_lower_mult = p.p2_lower_mult;
    c.p2_upper_mult = p.p2_upper_mult;
    return c;
}

void setErr(char* err, size_t len, const char* msg)
{
    if (err && len) {
        std::strncpy(err, msg, len - 1);
        err[len - 1] = 0;
    }
}

}  // namespace

extern "C" {

void pyrsgm_gb300_default_params(pyrsgm_gb300_params* p)
{
    if (p) *p = fromParams(pyrsgm::Params());
}

int pyrsgm_gb300_validate_params(const pyrsgm_gb300_params* in, pyrsgm_gb300_params* out, char* err, size_t len)
{
    if (!in) return -1;
    try {
        const pyrsgm::Params v = pyrsgm::validateParams(toParams(*in));
        if (out) *out = fromParams(v);
        return 0;
    } catch (const std::exception& e) {
        setErr(err, len, e.what());
        return -1;
    }
}

void* pyrsgm_gb300_matcher_create(int width, int height, const pyrsgm_gb300_params* p, char* err, size_t len)
{
    if (!p) return nullptr;
    try {
        return new pyrsgm::StereoMatcher(width, height, toParams(*p));
    } catch (const std::exception& e) {
        setErr(err, len, e.what());
        return nullptr;
    }
}

void pyrsgm_gb300_matcher_destroy(void* m) { delete static_cast<pyrsgm::StereoMatcher*>(m); }

int pyrsgm_gb300_matcher_compute(void* m, const unsigned char* L, size_t lp, const unsigned char* R, size_t rp,
                                 short* d16, size_t d16p, float* d32, size_t d32p, float* c, size_t cp,
                                 cudaStream_t st, char* err, size_t len)
{
    if (!m) return -1;
    try {
        static_cast<pyrsgm::StereoMatcher*>(m)->compute(L, lp, R, rp, d16, d16p, d32, d32p, c, cp, st);
        return 0;
    } catch (const std::exception& e) {
        setErr(err, len, e.what());
        return -1;
    }
}

int pyrsgm_gb300_matcher_level_info(void* m, int level, int* out7)
{
    if (!m || !out7) return -1;
    try {
        const pyrsgm::LevelInfo li = static_cast<pyrsgm::StereoMatcher*>(m)->levelInfo(level);
        out7[0] = li.level; out7[1] = li.width; out7[2] = li.height; out7[3] = li.num_labels;
        out7[4] = li.max_disparity; out7[5] = li.block_size; out7[6] = li.refine ? 1 : 0;
        return 0;
    } catch (...) {
        return -1;
    }
}

int pyrsgm_gb300_level_geometry(int width, int height, const pyrsgm_gb300_params* p, int* out35, char* err,
                                size_t len)
{
    if (!p || !out35) return -1;
    try {
        if (width <= 0 || height <= 0) throw std::invalid_argument("pyrsgm: empty image size");
        const pyrsgm::Params v = pyrsgm::validateParams(toParams(*p));
        std::array<pyrsgm::LevelInfo, 5> info{};
        pyrsgm::levelGeometry(width, height, v, info);
        for (int l = 0; l <= v.pyramid_levels; ++l) {
            const pyrsgm::LevelInfo& li = info[l];
            int* o = out35 + 7 * l;
            o[0] = li.level; o[1] = li.width; o[2] = li.height; o[3] = li.num_labels;
            o[4] = li.max_disparity; o[5] = li.block_size; o[6] = li.refine ? 1 : 0;
        }
        return v.pyramid_levels + 1;
    } catch (const std::exception& e) {
        setErr(err, len, e.what());
        return -1;
    }
}

int pyrsgm_gb300_matcher_num_levels(void* m) { return m ? static_cast<pyrsgm::StereoMatcher*>(m)->numLevels() : -1; }

size_t pyrsgm_gb300_matcher_device_bytes(void* m)
{
    return m ? static_cast<pyrsgm::StereoMatcher*>(m)->deviceMemoryBytes() : 0;
}

}  // extern "C"
