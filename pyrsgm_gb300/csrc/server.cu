// server.cu -- continuous-batching stereo server.  No counterpart in the
// reference (one pair per blocking-free call, no request handling).
//
// Requests carry host images and host output buffers.  A scheduler thread
// forms a batch from whatever has arrived once one of the server's stream
// lanes is free and the kernels of the batch before are done, or at once
// when a full batch is queued (up to max_batch pairs and the lane's device
// budget),
// copies the inputs on the lane's stream, runs the lane's batch engine on
// the compute stream that all lanes share (after the inputs) and copies the
// outputs back on the lane's stream (after the kernels), all
// asynchronously; while one lane's batch computes, the next lane copies
// the requests that arrived meanwhile in and its previous outputs out.
// Kernels of different lanes never run side by side: measured on 1080p
// D=256 pairs, two batches computing at once on two streams ran at less
// than half the rate of the same batches one after the other.  Each lane has a
// completion thread that waits for its lane's event, hands the results to
// the callers' buffers, records the latency (submit -> results in host
// memory) and frees the lane, independently of the other lanes.
//
// Host buffers that the caller registered (pyrsgm_gb300_server_register,
// page-locked with cudaHostRegister) are copied by DMA directly; other
// buffers go through the lane's pinned staging with a host memcpy.
//
// Device memory stays resident: the lanes share one batch engine, whose
// pooled pair plans may use the whole budget, and each lane keeps a pool of
// input/output buffers per image size.  A request is admitted only if it
// fits a lane's share of the budget on its own; a batch is cut where the
// next request would push it past that share.  Failures are
// per request (status -1 with a message): an invalid request is refused at
// submission, a full queue refuses new requests, and a batch whose
// allocation or launch fails fails its own requests while the server keeps
// serving.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include "pair_plan.h"
#include "trace.h"
#include "pyrsgm/pyrsgm_gb300.h"

namespace pyrsgm {
Params validateParams(const Params& in);
}

namespace pg {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
    long long id = 0;
    pyrsgm_gb300_request r{};
    size_t bytes = 0;
    double t_submit = 0, t_done = 0;
    int status = 0;  // 0 pending, 1 done, -1 failed
    unsigned long long trace = 0;   // NVTX range submit -> completion
    std::string error;
};

// Device and pinned-host I/O buffers of one image size.
struct IOBuf {
    int w = 0, h = 0;
    unsigned char *dL = nullptr, *dR = nullptr, *hL = nullptr, *hR = nullptr;
    short* d16 = nullptr;
    float *d32 = nullptr, *dc = nullptr;
    short* h16 = nullptr;
    float *h32 = nullptr, *hc = nullptr;
    size_t device_bytes() const { return (size_t)w * h * (2 + 2 + 4 + 4); }
    void alloc(int W_, int H_)
    {
        w = W_;
        h = H_;
        const size_t px = (size_t)w * h;
        auto ok = [](cudaError_t e) {
            if (e != cudaSuccess) throw std::runtime_error(std::string("server buffers: ") + cudaGetErrorString(e));
        };
        ok(cudaMalloc(&dL, px));
        ok(cudaMalloc(&dR, px));
        ok(cudaMalloc(&d16, px * 2));
        ok(cudaMalloc(&d32, px * 4));
        ok(cudaMalloc(&dc, px * 4));
        ok(cudaHostAlloc(&hL, px, cudaHostAllocDefault));
        ok(cudaHostAlloc(&hR, px, cudaHostAllocDefault));
        ok(cudaHostAlloc(&h16, px * 2, cudaHostAllocDefault));
        ok(cudaHostAlloc(&h32, px * 4, cudaHostAllocDefault));
        ok(cudaHostAlloc(&hc, px * 4, cudaHostAllocDefault));
    }
    void release()
    {
        for (void* p : {(void*)dL, (void*)dR, (void*)d16, (void*)d32, (void*)dc})
            if (p) cudaFree(p);
        for (void* p : {(void*)hL, (void*)hR, (void*)h16, (void*)h32, (void*)hc})
            if (p) cudaFreeHost(p);
        dL = dR = hL = hR = nullptr;
        d16 = h16 = nullptr;
        d32 = dc = h32 = hc = nullptr;
    }
};

class BatchEngine;
BatchEngine* batch_engine_new(size_t budget);
void batch_engine_delete(BatchEngine* e);
bool batch_engine_run(BatchEngine* e, const pyrsgm_gb300_pair* pairs, int n, cudaStream_t st, bool use_graph);
void batch_engine_reserve(BatchEngine* e, int w, int h, const pyrsgm::Params& p, int count, cudaStream_t st);

struct Lane {
    cudaStream_t st = nullptr;
    cudaEvent_t start = nullptr, done = nullptr;   // around the batch's GPU work (H2D .. D2H)
    cudaEvent_t inputs = nullptr, computed = nullptr;   // H2D finished; the batch's kernels finished
    double t_formed = 0, t_enqueued = 0;            // host clock: batch formed, all work enqueued
    std::map<std::pair<int, int>, std::vector<std::unique_ptr<IOBuf>>> pool;
    std::vector<Request*> reqs;
    std::vector<IOBuf*> bufs;
    std::vector<void*> staged;   // per request and output: staging used (null: copied in place or absent)
    bool busy = false;       // a batch is assigned to the lane and not yet finished
    bool computing = false;  // that batch's kernels have not finished yet
    bool launched = false;   // that batch is enqueued; the lane's completion thread takes it
    std::string error;  // set when the batch failed before reaching the GPU
    bool graph = false;  // the batch's kernels came from a captured graph
};

class Server {
public:
    Server(size_t budget, int max_batch, int lanes, int max_queue)
        : max_batch_(std::max(1, max_batch)), max_queue_(std::max(1, max_queue))
    {
        const int n = std::max(1, lanes);
        lane_budget_ = budget / n;
        if (cudaStreamCreateWithFlags(&cst_, cudaStreamNonBlocking) != cudaSuccess)
            throw std::runtime_error("server: stream creation failed");
        // one engine (one pool of pair plans) for all lanes: their kernels
        // run one batch after another on the compute stream, so a plan is
        // never used by two batches at once
        eng_ = batch_engine_new(budget);
        for (int i = 0; i < n; ++i) {
            auto L = std::make_unique<Lane>();
            if (cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreate(&L->start) != cudaSuccess || cudaEventCreate(&L->done) != cudaSuccess ||
                cudaEventCreate(&L->inputs) != cudaSuccess || cudaEventCreate(&L->computed) != cudaSuccess)
                throw std::runtime_error("server: stream/event creation failed");
            lanes_.push_back(std::move(L));
        }
        sched_ = std::thread([this] { schedule(); });
        // one completion thread per lane: a lane is free again as soon as its
        // own batch is done, whatever the other lanes are running
        for (auto& L : lanes_) comps_.emplace_back([this, l = L.get()] { complete(*l); });
    }

    ~Server()
    {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        sched_.join();
        for (auto& t : comps_) t.join();
        for (auto& L : lanes_) {
            cudaStreamSynchronize(L->st);
            for (auto& kv : L->pool)
                for (auto& b : kv.second) b->release();
            cudaEventDestroy(L->start);
            cudaEventDestroy(L->done);
            cudaEventDestroy(L->inputs);
            cudaEventDestroy(L->computed);
            cudaStreamDestroy(L->st);
        }
        cudaStreamSynchronize(cst_);
        batch_engine_delete(eng_);
        cudaStreamDestroy(cst_);
        for (auto& kv : reg_) cudaHostUnregister(reinterpret_cast<void*>(kv.first));
    }

    long long submit(const pyrsgm_gb300_request& r, std::string& err)
    {
        if (r.width <= 0 || r.height <= 0 || !r.h_left || !r.h_right) {
            err = "invalid request: empty size or null image";
            return -1;
        }
        pyrsgm::Params v;
        try {
            v = pyrsgm::validateParams(toParams(r.params));
        } catch (const std::exception& e) {
            err = std::string("invalid request: ") + e.what();
            return -1;
        }
        auto q = std::make_unique<Request>();
        q->r = r;
        q->bytes = PairPlan::bytesFor(r.width, r.height, v) + (size_t)r.width * r.height * 12;
        if (q->bytes > lane_budget_) {
            err = "request needs " + std::to_string(q->bytes) + " device bytes, more than a lane's budget (" +
                  std::to_string(lane_budget_) + ")";
            return -1;
        }
        std::lock_guard<std::mutex> lk(mu_);
        if ((int)queue_.size() >= max_queue_) {
            err = "queue full";
            ++refused_;
            return -1;
        }
        q->id = next_id_++;
        q->t_submit = now_s();
        q->trace = trace_start("pyrsgm.request");
        if (first_submit_ == 0) first_submit_ = q->t_submit;
        Request* raw = q.get();
        all_[raw->id] = std::move(q);
        queue_.push_back(raw);
        cv_.notify_all();
        return raw->id;
    }

    // 1 done, -1 failed (err set), 0 timed out.  A finished request is forgotten.
    int wait(long long id, double timeout_s, std::string& err)
    {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = all_.find(id);
        if (it == all_.end()) {
            err = "unknown request id";
            return -1;
        }
        Request* q = it->second.get();
        const auto pred = [&] { return q->status != 0; };
        if (timeout_s < 0) done_cv_.wait(lk, pred);
        else if (!done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return 0;
        const int s = q->status;
        err = q->error;
        all_.erase(it);
        return s;
    }

    // Wait until every submitted request finished; 1, or 0 on timeout.
    int drain(double timeout_s)
    {
        std::unique_lock<std::mutex> lk(mu_);
        const auto pred = [&] { return queue_.empty() && inflight_ == 0; };
        if (timeout_s < 0) {
            done_cv_.wait(lk, pred);
            return 1;
        }
        return done_cv_.wait_for(lk, std::chrono::duration<double>(timeout_s), pred) ? 1 : 0;
    }

    void stats(double* o)
    {
        std::lock_guard<std::mutex> lk(mu_);
        std::vector<double> l = lat_ms_;
        std::sort(l.begin(), l.end());
        auto pct = [&](double q) { return l.empty() ? 0.0 : l[std::min(l.size() - 1, (size_t)(q * (l.size() - 1) + 0.5))]; };
        o[0] = (double)ok_;
        o[1] = (double)failed_;
        o[2] = pct(0.50);
        o[3] = pct(0.99);
        o[4] = pct(0.999);
        o[5] = batches_ ? (double)batched_pairs_ / batches_ : 0.0;
        o[6] = (last_done_ > first_submit_ && ok_) ? ok_ / (last_done_ - first_submit_) : 0.0;
        o[7] = (double)max_inflight_pairs_;
        o[8] = (double)refused_;
        o[9] = l.empty() ? 0.0 : l.back();
    }

    // Mean per-stage times since the last reset: request wait in the queue,
    // host time to enqueue a batch (copies, kernels or graph replay), GPU
    // time of a batch (its H2D copies to its D2H copies, including time
    // spent waiting behind the other lanes' work), host time from the
    // batch's completion to its results in the callers' buffers; then the
    // batch count, the longest enqueue, the fraction of batches whose
    // kernels came from a captured graph, and the GPU time split into the
    // input copies, the kernels (with the wait for the compute stream) and
    // the output copies.
    void timeline(double* o)
    {
        std::lock_guard<std::mutex> lk(mu_);
        const double nb = tl_batches_ ? (double)tl_batches_ : 1.0;
        o[0] = tl_reqs_ ? tl_qwait_ms_ / tl_reqs_ : 0.0;
        o[1] = tl_enqueue_ms_ / nb;
        o[2] = tl_gpu_ms_ / nb;
        o[3] = tl_complete_ms_ / nb;
        o[4] = (double)tl_batches_;
        o[5] = tl_enqueue_max_ms_;
        o[6] = tl_batches_ ? (double)tl_graph_ / nb : 0.0;
        o[7] = tl_in_ms_ / nb;
        o[8] = tl_comp_ms_ / nb;
        o[9] = (tl_gpu_ms_ - tl_in_ms_ - tl_comp_ms_) / nb;
    }

    void reset_stats()
    {
        std::lock_guard<std::mutex> lk(mu_);
        tl_qwait_ms_ = tl_enqueue_ms_ = tl_gpu_ms_ = tl_complete_ms_ = tl_enqueue_max_ms_ = 0;
        tl_in_ms_ = tl_comp_ms_ = 0;
        tl_batches_ = tl_reqs_ = tl_graph_ = 0;
        lat_ms_.clear();
        ok_ = failed_ = refused_ = 0;
        batches_ = batched_pairs_ = 0;
        max_inflight_pairs_ = 0;
        first_submit_ = last_done_ = 0;
    }

    void inject_failure(int n)
    {
        std::lock_guard<std::mutex> lk(mu_);
        inject_ += n;
    }

    // Plans for `count` pairs of one shape in the shared engine, and device
    // and pinned I/O buffers for a full batch (max_batch pairs) of that size
    // on every lane, allocated now: batches of up to `count` such pairs then
    // allocate nothing (a cudaHostAlloc inside the stream stalls the
    // scheduler for milliseconds, and pairs of one size may fill a batch
    // whatever their parameters).
    int reserve(int w, int h, const pyrsgm_gb300_params& prm, int count, std::string& err)
    {
        try {
            const pyrsgm::Params p = toParams(prm);
            batch_engine_reserve(eng_, w, h, p, count, cst_);
            if (cudaStreamSynchronize(cst_) != cudaSuccess) throw std::runtime_error("reserve: stream error");
            std::lock_guard<std::mutex> lk(pool_mu_);
            for (auto& L : lanes_) {
                auto& vec = L->pool[{w, h}];
                while ((int)vec.size() < std::max(count, max_batch_)) {
                    vec.emplace_back(new IOBuf());
                    vec.back()->alloc(w, h);
                }
            }
            return 0;
        } catch (const std::exception& e) {
            err = e.what();
            return -1;
        }
    }

    // Page-lock a host range so that requests whose images or outputs lie
    // inside it are copied without staging.
    int register_host(void* p, size_t bytes, std::string& err)
    {
        if (!p || bytes == 0) {
            err = "null or empty range";
            return -1;
        }
        const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterDefault);
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = cudaGetErrorString(e);
            return -1;
        }
        std::lock_guard<std::mutex> lk(reg_mu_);
        reg_[reinterpret_cast<uintptr_t>(p)] = bytes;
        return 0;
    }

    // Only between requests that use the range (none in flight).
    int unregister_host(void* p)
    {
        {
            std::lock_guard<std::mutex> lk(reg_mu_);
            auto it = reg_.find(reinterpret_cast<uintptr_t>(p));
            if (it == reg_.end()) return -1;
            reg_.erase(it);
        }
        return cudaHostUnregister(p) == cudaSuccess ? 0 : -1;
    }

private:
    static pyrsgm::Params toParams(const pyrsgm_gb300_params& c)
    {
        pyrsgm::Params p;
        p.num_disparities = c.num_disparities;
        p.min_disparity = c.min_disparity;
        p.block_size = c.block_size;
        p.cost_mode = c.cost_mode == 1 ? pyrsgm::CostMode::Census : pyrsgm::CostMode::BirchfieldTomasi;
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

    // Whether a host range can be copied by DMA in place: registered with
    // this server, or page-locked by the caller (cudaHostAlloc /
    // cudaHostRegister elsewhere; its start and end both page-locked host
    // memory of the same allocation).
    bool registered(const void* p, size_t bytes)
    {
        const uintptr_t a = reinterpret_cast<uintptr_t>(p);
        {
            std::lock_guard<std::mutex> lk(reg_mu_);
            auto it = reg_.upper_bound(a);
            if (it != reg_.begin()) {
                --it;
                if (a >= it->first && a + bytes <= it->first + it->second) return true;
            }
        }
        cudaPointerAttributes at{}, bt{};
        if (cudaPointerGetAttributes(&at, p) != cudaSuccess ||
            cudaPointerGetAttributes(&bt, static_cast<const unsigned char*>(p) + bytes - 1) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return at.type == cudaMemoryTypeHost && bt.type == cudaMemoryTypeHost && at.hostPointer && bt.hostPointer &&
               static_cast<const unsigned char*>(bt.hostPointer) - static_cast<const unsigned char*>(at.hostPointer) ==
                   (ptrdiff_t)(bytes - 1);
    }

    IOBuf* take_buf(Lane& L, int w, int h, std::map<std::pair<int, int>, int>& used)
    {
        std::lock_guard<std::mutex> lk(pool_mu_);
        auto& vec = L.pool[{w, h}];
        int& k = used[{w, h}];
        if ((int)vec.size() <= k) {
            vec.emplace_back(new IOBuf());
            vec.back()->alloc(w, h);
        }
        return vec[k++].get();
    }

    // Scheduler: whenever a lane is free and requests are queued, launch a batch.
    void schedule()
    {
        for (;;) {
            Lane* L = nullptr;
            std::vector<Request*> batch;
            bool fail_batch = false;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] {
                    if (stop_) return true;
                    if (queue_.empty()) return false;
                    // a batch is formed once no earlier batch is still computing
                    // (what arrives meanwhile joins it instead of waiting behind
                    // it in a small batch of its own), or at once when a full
                    // batch is queued: then its input copies overlap the
                    // kernels before it, and its kernels follow them on the
                    // compute stream
                    bool computing = false;
                    for (auto& l : lanes_) computing = computing || l->computing;
                    if (computing && (int)queue_.size() < max_batch_) return false;
                    for (auto& l : lanes_)
                        if (!l->busy) return true;
                    return false;
                });
                if (stop_ && queue_.empty()) return;
                for (auto& l : lanes_)
                    if (!l->busy) { L = l.get(); break; }
                if (!L) continue;
                L->computing = true;
                size_t bytes = 0;
                while (!queue_.empty() && (int)batch.size() < max_batch_ && bytes + queue_.front()->bytes <= lane_budget_) {
                    bytes += queue_.front()->bytes;
                    batch.push_back(queue_.front());
                    queue_.pop_front();
                }
                L->busy = true;
                L->t_formed = now_s();
                for (Request* q : batch) tl_qwait_ms_ += (L->t_formed - q->t_submit) * 1e3;
                tl_reqs_ += (long long)batch.size();
                inflight_ += (int)batch.size();
                max_inflight_pairs_ = std::max(max_inflight_pairs_, (long long)inflight_);
                ++batches_;
                batched_pairs_ += (long long)batch.size();
                if (inject_ > 0) {
                    --inject_;
                    fail_batch = true;
                }
            }
            // canonical order (by shape): the same mix of shapes gets the same
            // buffers and plans, so the engine's graph of that mix replays
            std::stable_sort(batch.begin(), batch.end(), [](const Request* a, const Request* b) {
                return shape_key(a->r) < shape_key(b->r);
            });
            L->reqs = batch;
            L->bufs.clear();
            L->staged.clear();
            L->error.clear();
            try {
                if (fail_batch) throw std::runtime_error("injected allocation failure");
                launch(*L);
            } catch (const std::exception& e) {
                L->error = e.what();
                cudaGetLastError();
            }
            cudaEventRecord(L->done, L->st);
            L->t_enqueued = now_s();
            {
                std::lock_guard<std::mutex> lk(mu_);
                const double ms = (L->t_enqueued - L->t_formed) * 1e3;
                tl_enqueue_ms_ += ms;
                tl_enqueue_max_ms_ = std::max(tl_enqueue_max_ms_, ms);
                L->launched = true;
            }
            cv_.notify_all();
        }
    }

    static std::vector<long long> shape_key(const pyrsgm_gb300_request& r)
    {
        const pyrsgm_gb300_params& p = r.params;
        return {r.width, r.height, p.num_disparities, p.pyramid_levels, p.cost_mode, p.min_disparity, p.block_size,
                p.p1, p.p2, p.uniqueness_ratio, p.disp12_max_diff, p.lr_check, p.median_filter, p.num_paths,
                p.pre_filter_cap, p.pyramid_coarse_disparities, p.pyramid_max_disparity, p.adaptive_p2,
                (long long)(r.h_disp16 != nullptr), (long long)(r.h_disp32 != nullptr),
                (long long)(r.h_conf != nullptr)};
    }

    void launch(Lane& L)
    {
        TraceRange tr("pyrsgm.server.batch %d pairs", (int)L.reqs.size());
        std::map<std::pair<int, int>, int> used;
        std::vector<pyrsgm_gb300_pair> pairs;
        cudaEventRecord(L.start, L.st);
        for (Request* q : L.reqs) {
            const pyrsgm_gb300_request& r = q->r;
            IOBuf* b = take_buf(L, r.width, r.height, used);
            L.bufs.push_back(b);
            const size_t px = (size_t)r.width * r.height;
            const void* srcL = r.h_left;
            const void* srcR = r.h_right;
            if (!registered(srcL, px)) {
                std::memcpy(b->hL, r.h_left, px);
                srcL = b->hL;
            }
            if (!registered(srcR, px)) {
                std::memcpy(b->hR, r.h_right, px);
                srcR = b->hR;
            }
            if (cudaMemcpyAsync(b->dL, srcL, px, cudaMemcpyHostToDevice, L.st) != cudaSuccess ||
                cudaMemcpyAsync(b->dR, srcR, px, cudaMemcpyHostToDevice, L.st) != cudaSuccess)
                throw std::runtime_error("input copy failed");
            pyrsgm_gb300_pair p{};
            p.d_left = b->dL;
            p.left_pitch = r.width;
            p.d_right = b->dR;
            p.right_pitch = r.width;
            p.d_disp16 = r.h_disp16 ? b->d16 : nullptr;
            p.disp16_pitch = (size_t)r.width * 2;
            p.d_disp32 = r.h_disp32 ? b->d32 : nullptr;
            p.disp32_pitch = (size_t)r.width * 4;
            p.d_conf = r.h_conf ? b->dc : nullptr;
            p.conf_pitch = (size_t)r.width * 4;
            p.width = r.width;
            p.height = r.height;
            p.params = r.params;
            pairs.push_back(p);
        }
        // the kernels of every lane run on the one compute stream, after this
        // lane's inputs have arrived; the outputs are copied back on the
        // lane's stream once they are computed (lanes overlap copies with
        // each other's kernels, never kernels with kernels)
        if (cudaEventRecord(L.inputs, L.st) != cudaSuccess || cudaStreamWaitEvent(cst_, L.inputs, 0) != cudaSuccess)
            throw std::runtime_error("input event failed");
        L.graph = batch_engine_run(eng_, pairs.data(), (int)pairs.size(), cst_, true);
        if (cudaEventRecord(L.computed, cst_) != cudaSuccess || cudaStreamWaitEvent(L.st, L.computed, 0) != cudaSuccess)
            throw std::runtime_error("compute event failed");
        for (size_t i = 0; i < L.reqs.size(); ++i) {
            const pyrsgm_gb300_request& r = L.reqs[i]->r;
            IOBuf* b = L.bufs[i];
            const size_t px = (size_t)r.width * r.height;
            // outputs in registered memory land in place; the others in staging
            auto out = [&](void* user, void* stage, const void* dev, size_t n) {
                if (!user) {
                    L.staged.push_back(nullptr);
                    return;
                }
                const bool direct = registered(user, n);
                cudaMemcpyAsync(direct ? user : stage, dev, n, cudaMemcpyDeviceToHost, L.st);
                L.staged.push_back(direct ? nullptr : stage);
            };
            out(r.h_disp16, b->h16, b->d16, px * 2);
            out(r.h_disp32, b->h32, b->d32, px * 4);
            out(r.h_conf, b->hc, b->dc, px * 4);
        }
    }

    // Completion of one lane's batches (each lane has its own thread).
    void complete(Lane& lane)
    {
        Lane* L = &lane;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return L->launched || (stop_ && queue_.empty() && !L->busy); });
                if (!L->launched) return;
            }
            // the next batch may form as soon as this one's kernels are done
            // (its output copies overlap the next batch's input copies)
            if (L->error.empty()) cudaEventSynchronize(L->computed);
            {
                std::lock_guard<std::mutex> lk(mu_);
                L->computing = false;
            }
            cv_.notify_all();
            const cudaError_t e = cudaEventSynchronize(L->done);
            const double t_gpu = now_s();
            std::string err = L->error;
            float gpu_ms = 0.0f, in_ms = 0.0f, comp_ms = 0.0f;
            if (err.empty() && e == cudaSuccess &&
                (cudaEventElapsedTime(&gpu_ms, L->start, L->done) != cudaSuccess ||
                 cudaEventElapsedTime(&in_ms, L->start, L->inputs) != cudaSuccess ||
                 cudaEventElapsedTime(&comp_ms, L->inputs, L->computed) != cudaSuccess)) {
                cudaGetLastError();
                gpu_ms = in_ms = comp_ms = 0.0f;
            }
            if (err.empty() && e != cudaSuccess) err = cudaGetErrorString(e);
            if (err.empty()) {
                const cudaError_t e2 = cudaStreamQuery(L->st);
                if (e2 != cudaSuccess && e2 != cudaErrorNotReady) err = cudaGetErrorString(e2);
            }
            for (size_t i = 0; i < L->reqs.size() && err.empty(); ++i) {
                const pyrsgm_gb300_request& r = L->reqs[i]->r;
                IOBuf* b = L->bufs[i];
                const size_t px = (size_t)r.width * r.height;
                const void* const* st = &L->staged[3 * i];
                if (r.h_disp16 && st[0]) std::memcpy(r.h_disp16, b->h16, px * 2);
                if (r.h_disp32 && st[1]) std::memcpy(r.h_disp32, b->h32, px * 4);
                if (r.h_conf && st[2]) std::memcpy(r.h_conf, b->hc, px * 4);
            }
            const double t = now_s();
            {
                std::lock_guard<std::mutex> lk(mu_);
                for (Request* q : L->reqs) {
                    q->t_done = t;
                    trace_end(q->trace);
                    if (err.empty()) {
                        q->status = 1;
                        ++ok_;
                        lat_ms_.push_back((t - q->t_submit) * 1e3);
                        last_done_ = t;
                    } else {
                        q->status = -1;
                        q->error = err;
                        ++failed_;
                    }
                }
                inflight_ -= (int)L->reqs.size();
                if (err.empty()) {
                    ++tl_batches_;
                    tl_gpu_ms_ += gpu_ms;
                    tl_in_ms_ += in_ms;
                    tl_comp_ms_ += comp_ms;
                    tl_complete_ms_ += (t - t_gpu) * 1e3;
                    if (L->graph) ++tl_graph_;
                }
                L->reqs.clear();
                L->launched = false;
                L->busy = false;
            }
            done_cv_.notify_all();
            cv_.notify_all();
        }
    }

    const int max_batch_, max_queue_;
    cudaStream_t cst_ = nullptr;   // compute stream shared by the lanes
    BatchEngine* eng_ = nullptr;   // pair plans and graphs shared by the lanes
    std::mutex reg_mu_;
    std::mutex pool_mu_;   // the lanes' I/O buffer pools (scheduler and reserve())
    std::map<uintptr_t, size_t> reg_;   // registered host ranges: start -> bytes
    size_t lane_budget_ = 0;
    std::vector<std::unique_ptr<Lane>> lanes_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<Request*> queue_;

    std::unordered_map<long long, std::unique_ptr<Request>> all_;
    long long next_id_ = 0;
    int inflight_ = 0;
    bool stop_ = false;
    int inject_ = 0;
    std::vector<double> lat_ms_;
    double tl_qwait_ms_ = 0, tl_enqueue_ms_ = 0, tl_gpu_ms_ = 0, tl_complete_ms_ = 0, tl_enqueue_max_ms_ = 0;
    double tl_in_ms_ = 0, tl_comp_ms_ = 0;
    long long tl_batches_ = 0, tl_reqs_ = 0, tl_graph_ = 0;
    long long ok_ = 0, failed_ = 0, refused_ = 0, batches_ = 0, batched_pairs_ = 0, max_inflight_pairs_ = 0;
    double first_submit_ = 0, last_done_ = 0;
    std::thread sched_;
    std::vector<std::thread> comps_;
};

}  // namespace pg

namespace {
void setErr(char* err, size_t len, const std::string& msg)
{
    if (err && len) {
        std::strncpy(err, msg.c_str(), len - 1);
        err[len - 1] = 0;
    }
}
}  // namespace

extern "C" {

void* pyrsgm_gb300_server_create(size_t device_budget_bytes, int max_batch, int num_streams, int max_queue, char* err,
                                 size_t err_len)
{
    try {
        return new pg::Server(device_budget_bytes, max_batch, num_streams, max_queue);
    } catch (const std::exception& e) {
        setErr(err, err_len, e.what());
        return nullptr;
    }
}

void pyrsgm_gb300_server_destroy(void* s) { delete static_cast<pg::Server*>(s); }

long long pyrsgm_gb300_server_submit(void* s, const pyrsgm_gb300_request* r, char* err, size_t err_len)
{
    if (!s || !r) return -1;
    std::string e;
    const long long id = static_cast<pg::Server*>(s)->submit(*r, e);
    if (id < 0) setErr(err, err_len, e);
    return id;
}

int pyrsgm_gb300_server_wait(void* s, long long id, double timeout_s, char* err, size_t err_len)
{
    if (!s) return -1;
    std::string e;
    const int r = static_cast<pg::Server*>(s)->wait(id, timeout_s, e);
    if (r < 0) setErr(err, err_len, e);
    return r;
}

int pyrsgm_gb300_server_drain(void* s, double timeout_s) { return s ? static_cast<pg::Server*>(s)->drain(timeout_s) : -1; }

int pyrsgm_gb300_server_stats(void* s, double* out10)
{
    if (!s || !out10) return -1;
    static_cast<pg::Server*>(s)->stats(out10);
    return 0;
}

int pyrsgm_gb300_server_timeline(void* s, double* out10)
{
    if (!s || !out10) return -1;
    static_cast<pg::Server*>(s)->timeline(out10);
    return 0;
}

void pyrsgm_gb300_server_reset_stats(void* s)
{
    if (s) static_cast<pg::Server*>(s)->reset_stats();
}

int pyrsgm_gb300_server_inject_failure(void* s, int batches)
{
    if (!s) return -1;
    static_cast<pg::Server*>(s)->inject_failure(batches);
    return 0;
}

int pyrsgm_gb300_server_register(void* s, void* host, size_t bytes, char* err, size_t err_len)
{
    if (!s) {
        setErr(err, err_len, "null server");
        return -1;
    }
    std::string e;
    const int r = static_cast<pg::Server*>(s)->register_host(host, bytes, e);
    if (r != 0) setErr(err, err_len, e);
    return r;
}

int pyrsgm_gb300_server_reserve(void* s, int width, int height, const pyrsgm_gb300_params* params, int count,
                                char* err, size_t err_len)
{
    if (!s || !params) {
        setErr(err, err_len, "null server or params");
        return -1;
    }
    std::string e;
    const int r = static_cast<pg::Server*>(s)->reserve(width, height, *params, count, e);
    if (r != 0) setErr(err, err_len, e);
    return r;
}

int pyrsgm_gb300_server_unregister(void* s, void* host)
{
    return s ? static_cast<pg::Server*>(s)->unregister_host(host) : -1;
}

}  // extern "C"
