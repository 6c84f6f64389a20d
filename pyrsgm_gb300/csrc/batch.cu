// batch.cu -- many stereo pairs of different sizes, label counts, cost
// types and pyramid depths per launch.  No counterpart in the reference,
// which runs one pair per call with ~17 launches per level
// (src/sgm_kernels.cu:1617-1862); here the same per-pair results come from
// one launch per stage and kernel variant for the whole batch:
//
//   pyrDown     level k of every pair (both views), up to 32 images a launch
//   round r     level L_p - r of every pair p (coarsest first): features,
//               refine labels, cost (by cost type / refine), T->B and row pass
//               (by path-kernel shape), post -- up to 16 level jobs a launch
//
// Device memory: one PairPlan arena per pair slot, pooled by shape
// (width, height, validated parameters) and reused across runs; a run that
// would exceed the engine's byte budget fails before touching the GPU.
// CUDA graphs: a run whose signature (shapes, parameters, device pointers)
// matches a cached one replays that graph; a signature seen before but not
// cached is captured, instantiated and cached (32 signatures, least recently
// used dropped); a signature's first run is enqueued directly (with the
// autotuner, that run also measures the kernel shapes of its new launches).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "pair_plan.h"
#include "pyrsgm/pyrsgm_c.h"
#include "pyrsgm/pyrsgm_gb300.h"
#include "sgm_launch.h"
#include "trace.h"

namespace pyrsgm {
Params validateParams(const Params& in);
}

namespace pg {
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

// Pool key: everything that determines a plan's buffers and tables
// (field by field: the structs have padding bytes).
using ShapeKey = std::vector<long long>;

long long fbits(float f)
{
    unsigned u;
    std::memcpy(&u, &f, 4);
    return (long long)u;
}

ShapeKey keyOf(int w, int h, const pyrsgm::Params& v)
{
    return {w, h, v.num_disparities, v.min_disparity, v.block_size, (long long)v.cost_mode, v.p1, v.p2,
            v.uniqueness_ratio, v.disp12_max_diff, v.lr_check, v.median_filter, v.num_paths, v.pre_filter_cap,
            v.pyramid_levels, v.pyramid_coarse_disparities, v.pyramid_max_disparity, fbits(v.pyramid_min_confidence),
            v.adaptive_p2, fbits(v.p2_alpha), fbits(v.p2_beta), fbits(v.p2_lower_mult), fbits(v.p2_upper_mult)};
}

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("pyrsgm batch: ") + what + ": " + cudaGetErrorString(e));
}

struct Job {
    LevelDesc d;
    int level;
};

// Launch `stage` over jobs grouped by `key`, kBatchJobs at a time.
template <class KeyFn, class Stage>
void launchGrouped(std::vector<Job>& jobs, KeyFn key, Stage stage, cudaStream_t st, const char* what)
{
    std::stable_sort(jobs.begin(), jobs.end(), [&](const Job& a, const Job& b) { return key(a.d) < key(b.d); });
    size_t i = 0;
    while (i < jobs.size()) {
        size_t j = i;
        while (j < jobs.size() && key(jobs[j].d) == key(jobs[i].d)) ++j;
        for (size_t k = i; k < j; k += kBatchJobs) {
            Jobs<kBatchJobs> b;
            b.n = (int)std::min<size_t>(kBatchJobs, j - k);
            for (int q = 0; q < b.n; ++q) b.d[q] = jobs[k + q].d;
            check(stage(b, extent_of(b), st), what);
        }
        i = j;
    }
}

}  // namespace

class BatchEngine {
public:
    explicit BatchEngine(size_t budget) : budget_(budget) {}

    ~BatchEngine()
    {
        for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);
    }

    size_t bytesInUse() const { return used_; }

    // Pooled plans for `count` pairs of one shape, allocated now, so that
    // later runs with up to `count` such pairs allocate nothing.
    void reserve(int w, int h, const pyrsgm::Params& p, int count, cudaStream_t st)
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (w <= 0 || h <= 0 || count < 0) throw std::invalid_argument("pyrsgm: bad reserve request");
        const pyrsgm::Params v = pyrsgm::validateParams(p);
        const ShapeKey k = keyOf(w, h, v);
        auto& vec = pool_[k];
        const size_t each = PairPlan::bytesFor(w, h, v);
        while ((int)vec.size() < count) {
            if (used_ + each > budget_)
                throw std::runtime_error("pyrsgm batch: device-memory budget exceeded (" +
                                         std::to_string(used_ + each) + " > " + std::to_string(budget_) + " bytes)");
            vec.emplace_back(new PairPlan(w, h, v, st));
            used_ += vec.back()->arena_bytes;
        }
    }

    // True when the run's kernels came from a CUDA graph (replayed or just captured).
    bool run(const pyrsgm_gb300_pair* pairs, int n, cudaStream_t st, bool use_graph)
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (n <= 0) return false;
        std::vector<pyrsgm::Params> val(n);
        for (int i = 0; i < n; ++i) {
            const pyrsgm_gb300_pair& p = pairs[i];
            if (p.width <= 0 || p.height <= 0) throw std::invalid_argument("pyrsgm: empty image size");
            val[i] = pyrsgm::validateParams(toParams(p.params));
            if (!p.d_left || !p.d_right) throw std::invalid_argument("pyrsgm: null input image");
            if (p.d_disp16 && (p.disp16_pitch % 2) != 0)
                throw std::invalid_argument("pyrsgm: disp16 pitch must be even");
        }
        std::vector<PairPlan*> plans = acquire(pairs, val, n, st);
        std::vector<long long> sig = signature(pairs, val, n);
        if (st == nullptr || st == cudaStreamLegacy) use_graph = false;  // no capture on the legacy stream
        if (kChecked) use_graph = false;   // the checked build waits after every launch
        if (use_graph) {
            for (auto it = graphs_.begin(); it != graphs_.end(); ++it) {
                if (it->sig == sig) {
                    check(cudaGraphLaunch(it->exec, st), "graph launch");
                    count_launches(it->kernels);
                    it->last_use = ++tick_;
                    return true;
                }
            }
            cudaStreamCaptureStatus cs;
            check(cudaStreamIsCapturing(st, &cs), "capture status");
            if (cs != cudaStreamCaptureStatusNone) use_graph = false;  // caller is capturing: just enqueue
            // a signature is captured the second time it comes: batches of a
            // one-off composition (a server's mixed traffic) are enqueued
            // directly instead of paying for a capture and an instantiation
            if (use_graph && seen_[sig]++ == 0) {
                if (seen_.size() > 4096) seen_.clear();
                TuningScope scope;
                enqueue(pairs, plans, n, st);
                return false;
            }
        }
        if (!use_graph) {
            // measures unknown shape keys unless the stream is being captured
            TuningScope scope;
            enqueue(pairs, plans, n, st);
            return false;
        }
        cudaGraph_t g = nullptr;
        check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
        const unsigned long long n0 = launch_count();
        try {
            enqueue(pairs, plans, n, st);
        } catch (...) {
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        check(cudaStreamEndCapture(st, &g), "end capture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        check(e, "graph instantiate");
        if (graphs_.size() >= kMaxGraphs) {
            auto lru = std::min_element(graphs_.begin(), graphs_.end(),
                                        [](const Cached& a, const Cached& b) { return a.last_use < b.last_use; });
            cudaGraphExecDestroy(lru->exec);
            graphs_.erase(lru);
        }
        // the launches counted while capturing are the kernels this graph runs
        const unsigned long long kernels = launch_count() - n0;
        graphs_.push_back({std::move(sig), exec, ++tick_, kernels});
        check(cudaGraphLaunch(exec, st), "graph launch");
        return true;
    }

private:
    struct Cached {
        std::vector<long long> sig;
        cudaGraphExec_t exec;
        unsigned long long last_use;
        unsigned long long kernels;
    };
    static constexpr size_t kMaxGraphs = 32;

    // Plans for the pairs of one run: the i-th pair of a shape gets that
    // shape's i-th pooled plan (the same plans for the same batch).
    std::vector<PairPlan*> acquire(const pyrsgm_gb300_pair* pairs, const std::vector<pyrsgm::Params>& val, int n,
                                   cudaStream_t st)
    {
        std::map<ShapeKey, int> seen;
        size_t extra = 0;
        for (int i = 0; i < n; ++i) {
            const ShapeKey k = keyOf(pairs[i].width, pairs[i].height, val[i]);
            const int idx = seen[k]++;
            auto it = pool_.find(k);
            const size_t have = it == pool_.end() ? 0 : it->second.size();
            if ((size_t)idx >= have) extra += PairPlan::bytesFor(pairs[i].width, pairs[i].height, val[i]);
        }
        if (used_ + extra > budget_) {
            // release pooled plans of shapes this run does not use (cudaFree waits for the device)
            for (auto it = pool_.begin(); it != pool_.end() && used_ + extra > budget_;) {
                if (seen.count(it->first)) {
                    ++it;
                    continue;
                }
                for (auto& p : it->second) used_ -= p->arena_bytes;
                it = pool_.erase(it);
            }
            for (auto& g : graphs_) cudaGraphExecDestroy(g.exec);  // they may reference released plans
            graphs_.clear();
        }
        if (used_ + extra > budget_)
            throw std::runtime_error("pyrsgm batch: device-memory budget exceeded (" + std::to_string(used_ + extra) +
                                     " > " + std::to_string(budget_) + " bytes)");
        seen.clear();
        std::vector<PairPlan*> out(n);
        for (int i = 0; i < n; ++i) {
            const ShapeKey k = keyOf(pairs[i].width, pairs[i].height, val[i]);
            const int idx = seen[k]++;
            auto& vec = pool_[k];
            while ((int)vec.size() <= idx) {
                vec.emplace_back(new PairPlan(pairs[i].width, pairs[i].height, val[i], st));
                used_ += vec.back()->arena_bytes;
            }
            out[i] = vec[idx].get();
        }
        return out;
    }

    // Graph key: every field of every pair (pointers, pitches, shape,
    // parameters) and the kernel-form switches, so that a switch changed
    // after a capture takes effect on the next run.
    static std::vector<long long> signature(const pyrsgm_gb300_pair* pairs, const std::vector<pyrsgm::Params>& val,
                                            int n)
    {
        std::vector<long long> s;
        s.push_back(packed_words_override() * 100 + fused_mode() * 10 + tbw_mode());
        for (int i = 0; i < n; ++i) {
            const pyrsgm_gb300_pair& p = pairs[i];
            const long long f[] = {(long long)(uintptr_t)p.d_left, (long long)p.left_pitch,
                                   (long long)(uintptr_t)p.d_right, (long long)p.right_pitch,
                                   (long long)(uintptr_t)p.d_disp16, (long long)p.disp16_pitch,
                                   (long long)(uintptr_t)p.d_disp32, (long long)p.disp32_pitch,
                                   (long long)(uintptr_t)p.d_conf, (long long)p.conf_pitch};
            s.insert(s.end(), f, f + 10);
            const ShapeKey k = keyOf(p.width, p.height, val[i]);
            s.insert(s.end(), k.begin(), k.end());
        }
        return s;
    }

    void enqueue(const pyrsgm_gb300_pair* pairs, const std::vector<PairPlan*>& plans, int n, cudaStream_t st)
    {
        TraceRange tr("pyrsgm.batch %d pairs", n);
        int maxL = 0;
        for (int i = 0; i < n; ++i) maxL = std::max(maxL, plans[i]->levels);
        // pyramids, one level of every pair per launch group
        for (int level = 1; level <= maxL; ++level) {
            std::vector<PyrDownDesc> ds;
            int mw = 0, mh = 0;
            for (int i = 0; i < n; ++i) {
                const PairPlan& P = *plans[i];
                if (P.levels < level) continue;
                PyrDownDesc two[2];
                P.pyrdownDescs(level, pairs[i].d_left, pairs[i].left_pitch, pairs[i].d_right, pairs[i].right_pitch,
                               two);
                ds.push_back(two[0]);
                ds.push_back(two[1]);
                mw = std::max(mw, two[0].dw);
                mh = std::max(mh, two[0].dh);
            }
            for (size_t k = 0; k < ds.size(); k += kBatchPyr) {
                PyrDownBatch<kBatchPyr> b;
                b.n = (int)std::min<size_t>(kBatchPyr, ds.size() - k);
                for (int q = 0; q < b.n; ++q) b.d[q] = ds[k + q];
                check(launch_pyrdown(b, mw, mh, st), "pyrDown");
            }
        }
        // coarse-to-fine rounds
        for (int r = 0; r <= maxL; ++r) {
            std::vector<Job> jobs;
            for (int i = 0; i < n; ++i) {
                const PairPlan& P = *plans[i];
                const int level = P.levels - r;
                if (level < 0) continue;
                const pyrsgm_gb300_pair& q = pairs[i];
                if (!q.d_disp16 && !q.d_disp32 && !q.d_conf) continue;  // nothing requested
                LevelDesc d = level == 0 ? P.level0(q.d_left, q.left_pitch, q.d_right, q.right_pitch, q.d_disp16,
                                                    q.disp16_pitch, q.d_disp32, q.disp32_pitch, q.d_conf,
                                                    q.conf_pitch)
                                         : P.levelDesc(level);
                jobs.push_back({d, level});
            }
            if (jobs.empty()) continue;
            TraceRange tround("pyrsgm.round %d (%d level jobs)", r, (int)jobs.size());
            auto all = [](const LevelDesc&) { return 0; };
            launchGrouped(jobs, all, [](const Jobs<kBatchJobs>& b, const LevelExtent& e, cudaStream_t s) {
                return launch_prepare(b, e, s);
            }, st, "features");
            launchGrouped(jobs, [](const LevelDesc& d) { return d.cost * 2 + d.refine; },
                          [](const Jobs<kBatchJobs>& b, const LevelExtent& e, cudaStream_t s) {
                              return launch_cost(b, e, s);
                          }, st, "cost");
            launchGrouped(jobs, [](const LevelDesc& d) {
                return d.pyr * 100000 + path_variant(d.D);
            }, [](const Jobs<kBatchJobs>& b, const LevelExtent& e, cudaStream_t s) {
                return launch_paths(b, e, s);
            }, st, "aggregation");
            launchGrouped(jobs, all, [](const Jobs<kBatchJobs>& b, const LevelExtent& e, cudaStream_t s) {
                return launch_post(b, e, s);
            }, st, "post");
        }
    }

    std::mutex mu_;
    size_t budget_ = 0, used_ = 0;
    std::map<ShapeKey, std::vector<std::unique_ptr<PairPlan>>> pool_;
    std::vector<Cached> graphs_;
    std::map<std::vector<long long>, int> seen_;   // signatures run so far (uncaptured first runs)
    unsigned long long tick_ = 0;
};

BatchEngine* batch_engine_new(size_t budget) { return new BatchEngine(budget); }
void batch_engine_delete(BatchEngine* e) { delete e; }
bool batch_engine_run(BatchEngine* e, const pyrsgm_gb300_pair* pairs, int n, cudaStream_t st, bool use_graph)
{
    return e->run(pairs, n, st, use_graph);
}
void batch_engine_reserve(BatchEngine* e, int w, int h, const pyrsgm::Params& p, int count, cudaStream_t st)
{
    e->reserve(w, h, p, count, st);
}

}  // namespace pg

namespace {
void setErr(char* err, size_t len, const char* msg)
{
    if (err && len) {
        std::strncpy(err, msg, len - 1);
        err[len - 1] = 0;
    }
}
}  // namespace

extern "C" {

void* pyrsgm_gb300_batch_create(size_t device_budget_bytes, char* err, size_t err_len)
{
    try {
        return new pg::BatchEngine(device_budget_bytes);
    } catch (const std::exception& e) {
        setErr(err, err_len, e.what());
        return nullptr;
    }
}

void pyrsgm_gb300_batch_destroy(void* engine) { delete static_cast<pg::BatchEngine*>(engine); }

int pyrsgm_gb300_batch_run(void* engine, const pyrsgm_gb300_pair* pairs, int num_pairs, int use_graph,
                           cudaStream_t stream, char* err, size_t err_len)
{
    if (!engine || (num_pairs > 0 && !pairs)) return -1;
    try {
        static_cast<pg::BatchEngine*>(engine)->run(pairs, num_pairs, stream, use_graph != 0);
        return 0;
    } catch (const std::exception& e) {
        setErr(err, err_len, e.what());
        return -1;
    }
}

int pyrsgm_gb300_batch_reserve(void* engine, int width, int height, const pyrsgm_gb300_params* params, int count,
                               cudaStream_t stream, char* err, size_t err_len)
{
    if (!engine || !params) return -1;
    try {
        static_cast<pg::BatchEngine*>(engine)->reserve(width, height, pg::toParams(*params), count, stream);
        return 0;
    } catch (const std::exception& e) {
        setErr(err, err_len, e.what());
        return -1;
    }
}

size_t pyrsgm_gb300_batch_bytes_in_use(void* engine)
{
    return engine ? static_cast<pg::BatchEngine*>(engine)->bytesInUse() : 0;
}

size_t pyrsgm_gb300_pair_bytes(int width, int height, const pyrsgm_gb300_params* params)
{
    if (!params || width <= 0 || height <= 0) return 0;
    try {
        return pg::PairPlan::bytesFor(width, height, pyrsgm::validateParams(pg::toParams(*params)));
    } catch (...) {
        return 0;
    }
}

}  // extern "C"
