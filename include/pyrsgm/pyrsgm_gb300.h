/*
 * pyrsgm_gb300.h -- additions of pyrsgm-gb300 that have no counterpart in
 * the reference API: debug access to the internal volumes, a C surface over
 * pyrsgm::StereoMatcher, and sizing helpers.  Declarations here sit beside
 * the drop-in pyrsgm_c.h / pyrsgm.h, never instead of them.
 */
#ifndef PYRSGM_GB300_H
#define PYRSGM_GB300_H

#include <stddef.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Workspace debug flags. */
#define PYRSGM_GB300_DEBUG_AGGREGATED 1  /* keep the final aggregated cost volume in the workspace */

int pyrsgm_gb300_workspace_set_debug(void* workspace, int flags);

/* Device pointers to the workspace's matching-cost volume and aggregation
 * volume ([y][x][d] int16, d innermost, numDisparities labels) after the last
 * call on it.  The aggregation volume holds the final summed path costs only
 * when PYRSGM_GB300_DEBUG_AGGREGATED was set before that call. */
int pyrsgm_gb300_workspace_volumes(void* workspace, const short** cost, const short** aggregated,
                                   int* width, int* height, int* numDisparities);

/* Copy both volumes (width*height*numDisparities int16 each) into caller
 * device buffers (either may be NULL), asynchronously on `stream`. */
int pyrsgm_gb300_workspace_copy_volumes(void* workspace, short* cost, short* aggregated, cudaStream_t stream);

/* Device bytes one workspace of this geometry allocates. */
size_t pyrsgm_gb300_workspace_bytes(int width, int height, int numDisparities);

/* pyrsgm_compute_level without a workspace, for callers that may not
 * allocate device memory (hosts that own all device memory, real-time loops
 * where cudaMalloc's implicit synchronisation is not allowed).  No
 * counterpart in the reference.  Same arguments (minus the workspace),
 * results and return codes as pyrsgm_compute_level; the scratch is one
 * static 32 MiB device array, so a level must fit in it
 * (pyrsgm_gb300_workspace_bytes(width, height, numDisparities) <= 32 MiB,
 * e.g. 480x360 at 16 labels) or the call returns -1.  The first call on a
 * device looks up the array's device address (make it before any stream
 * capture) and keeps it for the life of the process: do not call it from a
 * context other than the device's primary context, nor after
 * cudaDeviceReset.  All calls share the array: calls whose GPU work
 * overlaps race and must be serialised by the caller. */
int pyrsgm_gb300_compute_level_noalloc(
    const unsigned char* d_left_gray, const unsigned char* d_right_gray,
    const short* d_parent_disp, const float* d_parent_conf,
    short* d_disp, float* d_disp_float, float* d_conf_float,
    size_t left_step_bytes, size_t right_step_bytes,
    size_t parent_disp_step_bytes, size_t parent_conf_step_bytes,
    size_t disp_step_bytes, size_t disp_float_step_bytes, size_t conf_float_step_bytes,
    int width, int height, int parent_width, int parent_height,
    int numDisparities, int minDisparity, int maxDisparity,
    int blockSize, int P1, int P2, int uniquenessRatio, int disp12MaxDiff,
    int preFilterCap, int costMode, int postFlags, int numPaths, int refineLevel,
    float minConfidence, int adaptiveP2,
    float p2Alpha, float p2Beta, float p2LowerMult, float p2UpperMult,
    cudaStream_t stream);

/* The adaptive-P2 table: d_table[i] (256 ints, device) = the effective P2 for
 * |I(p) - I(p-r)| = i, after the reference's parameter sanitising. */
int pyrsgm_gb300_p2_table(int* d_table, int P2, float p2Alpha, float p2Beta, float p2LowerMult, float p2UpperMult,
                          cudaStream_t stream);

/* pyrsgm::Params as a C struct (same fields, same defaults). */
typedef struct pyrsgm_gb300_params {
    int num_disparities, min_disparity, block_size, cost_mode;
    int p1, p2, uniqueness_ratio, disp12_max_diff;
    int lr_check, median_filter, num_paths, pre_filter_cap;
    int pyramid_levels, pyramid_coarse_disparities, pyramid_max_disparity;
    float pyramid_min_confidence;
    int adaptive_p2;
    float p2_alpha, p2_beta, p2_lower_mult, p2_upper_mult;
} pyrsgm_gb300_params;

void pyrsgm_gb300_default_params(pyrsgm_gb300_params* p);
/* pyrsgm::validateParams; returns 0, or -1 with the exception text in err. */
int pyrsgm_gb300_validate_params(const pyrsgm_gb300_params* in, pyrsgm_gb300_params* out, char* err,
                                 size_t err_len);

/* pyrsgm::StereoMatcher through C.  create returns NULL (message in err) on
 * failure; compute returns 0 or -1 (message in err). */
void* pyrsgm_gb300_matcher_create(int width, int height, const pyrsgm_gb300_params* p, char* err,
                                  size_t err_len);
void pyrsgm_gb300_matcher_destroy(void* matcher);
int pyrsgm_gb300_matcher_compute(void* matcher, const unsigned char* d_left, size_t left_pitch,
                                 const unsigned char* d_right, size_t right_pitch, short* d_disp16,
                                 size_t disp16_pitch, float* d_disp32, size_t disp32_pitch, float* d_conf,
                                 size_t conf_pitch, cudaStream_t stream, char* err, size_t err_len);
/* Level geometry of StereoMatcher(width, height, p) without allocating:
 * writes 7 ints per level (as pyrsgm_gb300_matcher_level_info) into out35
 * and returns the number of levels, or -1 (message in err). */
int pyrsgm_gb300_level_geometry(int width, int height, const pyrsgm_gb300_params* p, int* out35, char* err,
                                size_t err_len);
/* ---- Batched execution (no counterpart in the reference) ----------------
 * One stereo pair of a batch: device images and outputs as in
 * StereoMatcher::compute (outputs may be NULL; disp32 without conf uses a
 * scratch confidence), plus its own size and parameters. */
typedef struct pyrsgm_gb300_pair {
    const unsigned char* d_left;
    size_t left_pitch;
    const unsigned char* d_right;
    size_t right_pitch;
    short* d_disp16;
    size_t disp16_pitch;
    float* d_disp32;
    size_t disp32_pitch;
    float* d_conf;
    size_t conf_pitch;
    int width, height;
    pyrsgm_gb300_params params;
} pyrsgm_gb300_pair;

/* A batch engine owns pooled device memory (one arena per pair slot, reused
 * across runs) up to device_budget_bytes. */
void* pyrsgm_gb300_batch_create(size_t device_budget_bytes, char* err, size_t err_len);
void pyrsgm_gb300_batch_destroy(void* engine);
/* Enqueue all pairs on `stream`: every pyramid stage runs as one launch per
 * kernel variant for the whole batch.  Results equal StereoMatcher::compute
 * of each pair alone.  use_graph != 0: the run is captured as a CUDA graph
 * and replayed by later runs with the same pairs (pointers included); not on
 * the legacy default stream.  Returns 0, or -1 with the reason in err (bad
 * parameters, budget exceeded, CUDA error). */
int pyrsgm_gb300_batch_run(void* engine, const pyrsgm_gb300_pair* pairs, int num_pairs, int use_graph,
                           cudaStream_t stream, char* err, size_t err_len);
size_t pyrsgm_gb300_batch_bytes_in_use(void* engine);
/* Allocates now the pooled plans for `count` pairs of one shape (size and
 * parameters), so that later runs with up to `count` such pairs allocate
 * nothing; -1 with a message when the budget would be exceeded. */
int pyrsgm_gb300_batch_reserve(void* engine, int width, int height, const pyrsgm_gb300_params* params, int count,
                               cudaStream_t stream, char* err, size_t err_len);
/* Device bytes one pair of this size and parameters occupies in a batch
 * engine (or a StereoMatcher); 0 for invalid parameters. */
size_t pyrsgm_gb300_pair_bytes(int width, int height, const pyrsgm_gb300_params* params);

/* ---- Serving: continuous batching (no counterpart in the reference) -------
 * A request carries HOST images and HOST outputs (pitch = width; outputs may
 * be NULL).  The caller keeps the buffers alive until the request finished. */
typedef struct pyrsgm_gb300_request {
    const unsigned char* h_left;
    const unsigned char* h_right;
    short* h_disp16;
    float* h_disp32;
    float* h_conf;
    int width, height;
    pyrsgm_gb300_params params;
} pyrsgm_gb300_request;

/* num_streams lanes, each with its own copy stream and input/output
 * buffers; one batch engine (pooled pair plans within device_budget_bytes)
 * whose kernels run on one compute stream shared by the lanes; batches of
 * at most max_batch pairs and device_budget_bytes / num_streams of plans;
 * at most max_queue requests waiting. */
void* pyrsgm_gb300_server_create(size_t device_budget_bytes, int max_batch, int num_streams, int max_queue,
                                 char* err, size_t err_len);
void pyrsgm_gb300_server_destroy(void* server);
/* Request id (>= 0), or -1 with the reason in err (invalid request, larger
 * than a lane's budget, queue full).  Thread-safe. */
long long pyrsgm_gb300_server_submit(void* server, const pyrsgm_gb300_request* req, char* err, size_t err_len);
/* 1 = done (outputs written), -1 = failed (reason in err), 0 = timeout
 * (timeout_s < 0 waits forever).  A finished request's id is released. */
int pyrsgm_gb300_server_wait(void* server, long long id, double timeout_s, char* err, size_t err_len);
/* Wait until every submitted request finished: 1, or 0 on timeout. */
int pyrsgm_gb300_server_drain(void* server, double timeout_s);
/* out10 = completed, failed, latency p50 / p99 / p99.9 ms (submit -> outputs
 * in host memory), mean batch size, pairs/s (first submit -> last
 * completion), peak pairs in flight, refused submissions, max latency ms. */
int pyrsgm_gb300_server_stats(void* server, double* out10);
/* Where a request's time goes, as means since the last reset (out10[10]):
 * queue wait per request (submit -> batch formed), host time to enqueue a
 * batch, GPU time of a batch (its input copies to its output copies, waits
 * behind other lanes' work included), host time from a batch's completion to
 * the results in the callers' buffers (all ms); then the number of batches,
 * the longest enqueue (ms), the fraction of batches whose kernels came from a
 * captured CUDA graph, and the batch's GPU time split into input copies,
 * kernels (with the wait for the shared compute stream) and output copies
 * (ms). */
int pyrsgm_gb300_server_timeline(void* server, double* out10);
void pyrsgm_gb300_server_reset_stats(void* server);
/* Test hook: the next `batches` batches fail on the host before reaching the
 * GPU, as an allocation failure would; their requests report -1. */
int pyrsgm_gb300_server_inject_failure(void* server, int batches);
/* Page-lock a host range (cudaHostRegister): request images and outputs
 * that lie inside a registered range -- or in memory the caller page-locked
 * itself (cudaHostAlloc, cudaHostRegister) -- are copied by DMA in place,
 * the others through the server's pinned staging with a host memcpy.  0, or -1 with the
 * reason in err.  Unregister only while no request using it is in flight;
 * the server unregisters what is left when destroyed. */
int pyrsgm_gb300_server_register(void* server, void* host, size_t bytes, char* err, size_t err_len);
/* Plans for `count` pairs of one shape kept resident in the server's pool,
 * which all stream lanes share, and device and pinned input/output buffers
 * for a full batch (max_batch pairs) of that size on every lane (returns
 * when allocated): a server expecting bursts of one shape keeps that many
 * resident, so no request waits for an allocation. */
int pyrsgm_gb300_server_reserve(void* server, int width, int height, const pyrsgm_gb300_params* params, int count,
                                char* err, size_t err_len);
int pyrsgm_gb300_server_unregister(void* server, void* host);

/* out[7] = level, width, height, num_labels, max_disparity, block_size, refine */
int pyrsgm_gb300_matcher_level_info(void* matcher, int level, int* out7);
int pyrsgm_gb300_matcher_num_levels(void* matcher);
size_t pyrsgm_gb300_matcher_device_bytes(void* matcher);

const char* pyrsgm_gb300_version(void);

/* Kernel launches issued by this library since the process started. */
unsigned long long pyrsgm_gb300_launch_count(void);

/* 1 in the checked build (libpyrsgm_gb300_checked.so, compiled with
 * PYRSGM_CHECKED): there, chosen global-memory accesses of the kernels are
 * range-checked on the device (a failed check records its site and skips
 * the access), every launch is followed by a wait on its stream and an
 * error check, and the batch engine captures no graphs.  0 in the default
 * build. */
int pyrsgm_gb300_checked(void);
/* Failures the checked build has seen since load (launch errors and failed
 * range checks; the call that met one returned an error), with the first
 * one's description copied to `first` (may be NULL).  Always 0 in the
 * default build. */
int pyrsgm_gb300_check_report(char* first, size_t len);

/* Opt-in speckle filter on an int16 disparity map (device pointer, pitch in
 * bytes), enqueued on `stream`: 4-neighbours belong to one region when
 * neither equals new_val and their values differ by at most max_diff (in the
 * map's units, e.g. 16 per pixel for disparity x16); regions of at most
 * max_speckle_size pixels are set to new_val -- the semantics of OpenCV's
 * cv::filterSpeckles, which the reference's benchmark leaves off.  Not part
 * of compute(); max_speckle_size <= 0 does nothing.  Scratch of 8 bytes per
 * pixel comes from the stream-ordered allocator.  0, or -1 on bad arguments
 * or a failed allocation/launch. */
int pyrsgm_gb300_filter_speckles(short* d_disp, size_t pitch_bytes, int width, int height, short new_val,
                                 int max_speckle_size, int max_diff, cudaStream_t stream);

/* Shape of the 16/32/64-label aggregation kernels: 0 chooses per launch
 * (one thread per 16 labels when the launch has rows enough to fill the
 * GPU, else a chain spread over more threads), 8 forces the former, 2 or 4
 * the latter.  Results are identical either way.  Returns the previous
 * setting, or -1 for another value.  The environment variable
 * PYRSGM_GB300_PACKED_NW gives the initial setting. */
int pyrsgm_gb300_set_packed_words(int words);

/* Fused aggregation of the 16-label pyramid levels with three paths (off by
 * default; PYRSGM_GB300_FUSED=1 turns it on at load).  When on, the wide
 * shape of those levels is two passes -- top-to-bottom and left-to-right
 * together on a skewed front of 32-row bands (each band waits, bounded, for
 * the band above's bottom edge), then right-to-left with the
 * winner-take-all -- instead of three path passes and a winner-take-all
 * pass; results are identical.  Returns the previous setting. */
int pyrsgm_gb300_set_fused(int on);

/* Winner-take-all inside the top-to-bottom pass for the 16-label pyramid
 * levels with three paths, in the one-thread-per-16-labels shape: the row
 * pass runs first and the top-to-bottom chains add their costs to the row
 * paths' and pick the winners, instead of writing a top-to-bottom volume
 * for a separate winner-take-all pass.  Mode 1 (default) takes this form
 * for launches with columns for at least 9 warps per SM, where it is the
 * faster one; 0 never, 2 always.  PYRSGM_GB300_TBW gives the initial mode.
 * Results are identical.  Returns the previous mode, or -1 for another
 * value. */
int pyrsgm_gb300_set_tbw(int mode);

/* Waits of the fused pass that ran out of time (a band whose band above
 * never published its edge; results of that launch are wrong), counted on
 * the current device since load or the last reset.  Synchronous.
 * 0xffffffff if the count could not be read. */
unsigned pyrsgm_gb300_fused_stalls(int reset);

/* Measuring choice of that shape (off by default; the environment variable
 * PYRSGM_GB300_AUTOTUNE=1 turns it on at load).  When on, the first run of
 * a new batch in the batch engine (before its CUDA graph is captured)
 * times both shapes for every aggregation launch whose key -- label count,
 * pyramid mode, total rows, widest level -- has no entry yet, and records
 * the faster; later launches with that key use it.  Timing synchronises
 * the host with the stream, once per new key.  A forced shape
 * (pyrsgm_gb300_set_packed_words) takes precedence.  Returns the previous
 * setting. */
int pyrsgm_gb300_set_autotune(int on);

typedef struct {
    int num_labels, pyramid, rows, width;  /* key; pyramid: 0 single-scale, 1 pyramid level,
                                              2 with the fused passes, 3 with the T->B winner-take-all */
    int words;                             /* chosen words per thread (8, or 2/4) */
    float ms_wide, ms_spread;              /* best time of each shape */
} pyrsgm_gb300_tune_entry;

/* Copies up to `capacity` recorded entries to `out` (may be NULL) and
 * returns how many there are. */
int pyrsgm_gb300_autotune_entries(pyrsgm_gb300_tune_entry* out, int capacity);
/* Forgets every entry. */
void pyrsgm_gb300_autotune_clear(void);

/* Per-kernel profiling with CUDA events recorded on each launch's stream.
 * pyrsgm_gb300_profile(1) clears the records and starts recording,
 * pyrsgm_gb300_profile(0) stops.  _read() waits for the recorded events of
 * one kernel kind (0 pyrDown, 1 features, 2 refine labels, 3 cost volume,
 * 4 top->bottom path, 5 row pass, 6 post, 7 P2 table, 8 winner-take-all of
 * the 16/32/64-label levels, 9 and 10 the fused passes, 11 top->bottom with
 * the winner-take-all) and returns the summed
 * device time in ms, the launch count and the summed algorithmic bytes. */
int pyrsgm_gb300_profile(int enable);
int pyrsgm_gb300_profile_read(int kind, double* ms_total, long long* launches, double* bytes_total);

#ifdef __cplusplus
}
#endif

#endif /* PYRSGM_GB300_H */
