/*
 * sister_gb300 -- GB300 (sm_103a) implementation of SiSter's 5-view multiview disparity.
 *
 * C ABI of libsister_gb300.so. Plain pointers and sizes only. Every entry point returns a status
 * (SISTER_OK = 0 or a negative SISTER_E* code); sister_last_error() gives the message.
 *
 * Reference interface replaced (paths relative to the reference project root):
 *   class SisterMultiviewDisparities                     cpp/include/sister/SisterMultiviewDisparities.hpp:18
 *     ctor (center, right, top, left, bottom)            ...SisterMultiviewDisparities.hpp:22
 *     compute_disparities(dispCount, multi, horiz, vert) ...SisterMultiviewDisparities.hpp:26-119
 *   callers: cpp/src/compute_disp.cpp:26-35 and the ROS service recipe ros/README.md:47-56.
 *
 * Outputs follow the reference exactly: u16 images of the ORIGINAL size w x h holding disparity*255
 * (saturated at 65535), bit-exact with the reference CPU path on the same input. Inputs are 8-bit
 * images, either gray (channels = 1) or BGR (channels = 3, converted with OpenCV's published
 * fixed-point BGR2GRAY weights). Preconditions the reference leaves implicit are checked:
 * w % 4 == 0, h % 4 == 0, 8 <= dc <= 512, dc % 8 == 0.
 */
#ifndef SISTER_GB300_H
#define SISTER_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define SISTER_API __attribute__((visibility("default")))
#else
#define SISTER_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum {
    SISTER_OK = 0,
    SISTER_EINVAL = -1,   /* bad argument / unsupported geometry */
    SISTER_ENOMEM = -2,   /* device allocation failed */
    SISTER_EBUDGET = -3,  /* request exceeds the configured HBM budget (serving) */
    SISTER_EDEVICE = -4,  /* CUDA error */
    SISTER_ETIMEOUT = -5, /* a bounded device-side wait expired */
    SISTER_ESTATE = -6,   /* call order violated (e.g. compute before load) */
    SISTER_EBUSY = -7,    /* serving: the request queue is full; nothing was queued (retry later) */
    SISTER_EPENDING = -8  /* serving: the request is still queued or running (the ticket stays valid) */
};

typedef struct sister_ctx sister_ctx;

/* --- plain drop-in path (one rig at a time) -------------------------------------------------- */

/* Create a context on CUDA device `device`. Replaces constructing SisterMultiviewDisparities. */
SISTER_API int sister_ctx_create(sister_ctx **out, int device);
SISTER_API void sister_ctx_destroy(sister_ctx *ctx);
SISTER_API const char *sister_last_error(const sister_ctx *ctx);

/* Load the five views in the reference constructor's order {center, right, top, left, bottom}
 * (SisterMultiviewDisparities.hpp:22), each `height` rows of `width` pixels with row pitch `stride`
 * bytes, `channels` 1 (gray) or 3 (BGR, SisterMultiviewDisparities.hpp:29-33). Host pointers. */
SISTER_API int sister_load_views(sister_ctx *ctx, const uint8_t *const views[5], int width, int height, int stride,
                      int channels);
/* Same, with device pointers (images already resident in HBM). */
SISTER_API int sister_load_views_device(sister_ctx *ctx, const uint8_t *const views[5], int width, int height,
                             int stride, int channels);

/* The dispCount argument of compute_disparities (SisterMultiviewDisparities.hpp:26). */
SISTER_API int sister_set_max_disparity(sister_ctx *ctx, int dc);

/* compute_disparities (SisterMultiviewDisparities.hpp:26-119): writes width*height u16 images to host
 * buffers. `multi` is mode 0 (all four pairs), `horiz` mode 1, `vert` mode 2; any may be NULL and the
 * corresponding aggregation is then skipped. Blocks until the results are on the host. */
SISTER_API int sister_compute(sister_ctx *ctx, uint16_t *multi, uint16_t *horiz, uint16_t *vert);

/* Two-view stereo of the reference's doStereo (SisterMultiviewDisparities.hpp:122-150; dead code there, offered
 * here as the same pipeline for one image pair): census of both images, Hamming cost volume, the 8-path
 * aggregation, WTA-left and WTA-right, in-place 3x3 medians of both maps and the LR check (threshold 5), on the
 * images as given (no padding). center and other: host gray images (width x height, row stride `stride`), other
 * being the image searched at (y, x - d) like the multiview right view. Outputs (host, width*height each): left =
 * the checked left disparities, -10 where rejected (the reference's float map holds the same integers); right =
 * the median-filtered right map. Same size and dc rules as sister_compute. */
SISTER_API int sister_stereo(sister_ctx *ctx, const uint8_t *center, const uint8_t *other, int width, int height,
                             int stride, int dc, int16_t *left, uint16_t *right);
/* Same with device output pointers; asynchronous on the context stream (see sister_synchronize). */
SISTER_API int sister_compute_device(sister_ctx *ctx, uint16_t *multi, uint16_t *horiz, uint16_t *vert);

/* Use an external cudaStream_t (NULL restores the context's own stream). */
SISTER_API int sister_set_stream(sister_ctx *ctx, void *stream);
/* Wait for queued work; reports device-side errors (e.g. SISTER_ETIMEOUT) of completed launches. */
SISTER_API int sister_synchronize(sister_ctx *ctx);

/* Bytes of device memory the context would hold for one output mode of a w x h rig at max disparity dc (about
 * 4.6 GB for 1920x1080 at 256: the cost volume of (w+2dc)(h+2dc) pixels and the two pass sums of the w x h
 * original pixels, 32*ceil(dc/32) u16 each, dominate; SISTER_TUNE_FULL_DISP keeps sums of all padded pixels). */
SISTER_API size_t sister_device_bytes(int width, int height, int dc);

/* --- aggregation without device allocation ------------------------------------------------ */
/* No counterpart in the reference (which allocates every buffer per call with _mm_malloc).
 * For callers that cannot allocate device memory when they need a result -- a robot or ROS callback
 * with a fixed, pre-reserved memory budget and hard latency limits, or code inside a framework that owns
 * all device allocations. Runs the same 8-path aggregation, winner-take-all, crop and *255 as
 * sister_compute on a masked cost volume the caller already holds in device memory:
 *   cost   [(h+2dc)][(w+2dc)][dstride] u16, 16-byte aligned, entries d >= dc set to 0x7FFF (the layout
 *          SISTER_DBG_COST returns); dstride = 32*k for the smallest k in {2,4,6,8,12,16} with 32*k >= dc
 *   out    w x h u16 disparity*255 (device, may be NULL); disp_padded (h+2dc) x (w+2dc) u16 (device, may be NULL)
 * It calls no cudaMalloc/cudaFree: its scratch (pass sum, hand-off records, counters, error flag) lives in
 * one static device array of SISTER_STATIC_SCRATCH_BYTES that every GPU loading the library holds until
 * exit. Requests needing more return SISTER_EBUDGET with the sizes in `err`. The first call on each device
 * looks up that array's device address and sets kernel attributes (make that first call before any stream
 * capture). All calls share the array and it keeps the last call's contents; the call clears what must
 * start at zero. Calls that overlap on the GPU (other streams, other host threads) race on it. The call
 * runs on `stream` (NULL: legacy default stream) and returns once the results are written. */
#define SISTER_STATIC_SCRATCH_BYTES (32u << 20)
SISTER_API int sister_aggregate_static(const uint16_t *cost, int width, int height, int dc, int dstride, uint16_t *out,
                                       uint16_t *disp_padded, void *stream, char *err, size_t errlen);

/* --- stage profiling: CUDA events on the context stream around every stage ----------------- */
enum {
    SISTER_STAGE_FRAMES = 1,   /* padded, rotated frame images */
    SISTER_STAGE_CENSUS = 2,   /* 9x7 census of the eight frame images */
    SISTER_STAGE_PAIR_WTA = 3, /* per-pair WTA-left/right from census words and, in the same launch, the
                                  row-recursive 3x3 medians that follow the WTA rows */
    SISTER_STAGE_MASKS = 5,    /* LR check and confidence masks */
    SISTER_STAGE_COST = 6,     /* masked multiview cost volume (once per computed mode) */
    SISTER_STAGE_AGGREGATE = 7, /* 8-path aggregation, both passes concurrently, and the final winner-take-all,
                                   crop and *255 of every output row in the same launch (all computed modes) */
    SISTER_STAGE_WTA = 8        /* the final winner-take-all as its own kernel: only with SISTER_TUNE_FULL_DISP
                                   (the padded map); otherwise ~0 */
};
/* Enable/disable event recording for subsequent computes (no reference counterpart: the reference only
 * prints clock() around whole modes, SisterMultiviewDisparities.hpp:73-89). */
SISTER_API int sister_profile_enable(sister_ctx *ctx, int on);
/* Durations (ms) and stage ids of the last compute, in launch order; waits for its completion. */
SISTER_API int sister_profile_read(sister_ctx *ctx, float *ms, int *stage, int max, int *count);

/* --- tuning: launch-shape knobs of the aggregation kernels (0 = automatic) ------------------- */
enum {
    SISTER_TUNE_SGM_ROWS = 1,     /* image rows per CTA (one warp each); 0 = automatic */
    SISTER_TUNE_SGM_CLUSTER = 2,  /* CTAs per thread-block cluster (1, 2, 4 or 8); 0 = automatic */
    SISTER_TUNE_SGM_GROUPS = 3,   /* read-only: cluster-sized row groups of the current geometry */
    SISTER_TUNE_SGM_CLUSTERS = 4, /* read-only: co-resident clusters launched */
    SISTER_TUNE_FULL_DISP = 5,    /* 1: also write the padded winner-take-all map (SISTER_DBG_DISP) and keep the pass
                                     sums of the whole padded plane (SISTER_DBG_SUM0), with the final WTA as its own
                                     kernel; 0 (default): only the cropped outputs, pass sums of the original pixels,
                                     the final WTA inside the aggregation launch */
    SISTER_TUNE_WAIT_LIMIT_US = 6 /* longest device-side wait of one warp on another warp or CTA (band hand-offs,
                                     median row flags) before the kernel gives up, raises its error flag and
                                     finishes: the compute then returns SISTER_ETIMEOUT and the context stays
                                     usable. 0 = default (2 s). A small value makes waits expire on purpose
                                     (tests of the failure path). */
};
/* Set a knob for subsequent computes (no reference counterpart: the reference is single-threaded CPU code). */
SISTER_API int sister_tune_set(sister_ctx *ctx, int key, int value);
/* Read the value in effect for the current geometry (after set_max_disparity and load_views). */
SISTER_API int sister_tune_get(sister_ctx *ctx, int key, int *value);

/* --- batched rigs -------------------------------------------------------------------------------------
 * Throughput path for many independent rigs (no reference counterpart: the reference computes one rig per
 * SisterMultiviewDisparities object, hpp:18-26). Each rig is computed exactly as sister_compute would. */
typedef struct sister_rig {
    const uint8_t *views[5];   /* host images, reference constructor order: center, right, top, left, bottom */
    int width, height, stride; /* stride in bytes */
    int channels;              /* 1 (gray) or 3 (BGR) */
    int max_disparity;         /* dispCount: multiple of 8 in [8, 512] */
    uint16_t *multi, *horiz, *vert; /* host outputs, width*height u16 each (disparity*255); NULL skips a mode */
} sister_rig;
typedef struct sister_batch sister_batch;
/* budget_bytes: device memory the engine may hold, allocated here as one arena (0: three quarters of the
 * device's free memory). */
SISTER_API int sister_batch_create(sister_batch **out, int device, size_t budget_bytes);
SISTER_API void sister_batch_destroy(sister_batch *batch);
SISTER_API const char *sister_batch_last_error(sister_batch *batch);
/* Computes every rig and returns when all outputs are written. Rigs run in waves whose device memory fits the
 * budget; within a wave the stages before the aggregation run per rig on several streams, and one persistent
 * aggregation launch per disparity-stride class covers all of the wave's rigs and modes (work items ordered by
 * band, so one rig's wavefront ramp is filled with the others' bands). A bad rig, or one that alone exceeds the
 * budget, fails the call (SISTER_EINVAL / SISTER_EBUDGET) before anything runs. */
SISTER_API int sister_batch_run(sister_batch *batch, const sister_rig *rigs, int nrigs);
/* Device bytes one rig takes inside a batch when nmodes of its outputs are requested (each mode has its own
 * aggregation volumes, since a wave aggregates all of them in one launch; BGR input counted). */
SISTER_API size_t sister_batch_rig_bytes(int width, int height, int max_disparity, int nmodes);

/* --- serving loop ------------------------------------------------------------------------------------
 * Requests (one rig each: dispCount + five images -> disparity images, the request shape of the reference's
 * ROS service recipe, ros/README.md:6-15) are submitted from any host thread and served with continuous
 * admission: a request starts as soon as a stream slot is free and its device memory fits the budget beside the
 * requests already running (in arrival order), its stages overlap theirs on the device, and its ticket completes
 * when its own outputs are in host memory. The rig's views and outputs must stay valid until sister_server_wait
 * returns for its ticket. */
typedef struct sister_server sister_server;
SISTER_API int sister_server_create(sister_server **out, int device, size_t budget_bytes);
SISTER_API void sister_server_destroy(sister_server *server); /* finishes admitted and queued requests first */
/* Message of the last failure; the string belongs to the calling thread until its next call. */
SISTER_API const char *sister_server_last_error(sister_server *server);
/* Requests computed at once (1..16, default 8) and requests waiting for admission (default 1024). */
SISTER_API int sister_server_set_limits(sister_server *server, int max_inflight, size_t max_queue);
/* SISTER_EBUDGET if the rig alone exceeds the budget, SISTER_EBUSY if the queue is full (backpressure),
 * SISTER_EINVAL for a bad rig; nothing is queued then. */
SISTER_API int sister_server_submit(sister_server *server, const sister_rig *rig, uint64_t *ticket);
/* Blocks up to timeout_ms. Returns the request's status once its outputs are in host memory (the ticket is
 * then released; SISTER_ETIMEOUT means a device-side wait of that request expired) or SISTER_EPENDING if it is
 * still queued or running (the ticket stays valid). latency_ms: submission to outputs in host memory. Finished
 * tickets that are never waited for are dropped after 4096 later completions. */
SISTER_API int sister_server_wait(sister_server *server, uint64_t ticket, int timeout_ms, double *latency_ms);
/* Counters: requests admitted, completed, refused for a full queue, and the most requests in flight at once. */
SISTER_API int sister_server_stats(sister_server *server, uint64_t *admitted, uint64_t *completed, uint64_t *rejected,
                                   int *peak_inflight);

/* --- synthetic workloads ------------------------------------------------------------------------------
 * Seeded synthetic rig (no dataset ships with the reference): views = 5 x h x w u8 (center, right, top,
 * left, bottom), disparity = h x w (may be NULL). Byte-identical to sister_gb300/synth.py make_rig;
 * sigma_tenths 15 or 8 (texture blur). Host only. */
SISTER_API int sister_synth_rig(int width, int height, int dmin, int dmax, long long seed, int tiles, int bump,
                                int sigma_tenths, uint8_t *views, int32_t *disparity);

/* --- test hooks: intermediates of the last compute (device -> host copies) -------------------- */
enum {
    SISTER_DBG_FRAMES = 1, /* index k=0..7: frame image k (u8) */
    SISTER_DBG_CENSUS = 2, /* index k=0..7: census of frame image k (u64) */
    SISTER_DBG_WTA = 3,    /* index 2f / 2f+1: WTA-left / WTA-right of frame f before the median (u16) */
    SISTER_DBG_MEDIAN = 4, /* index 2f / 2f+1: after the in-place median (u16) */
    SISTER_DBG_MASKS = 5,  /* index f: confidence mask of frame f in padded original coordinates (u8) */
    SISTER_DBG_COST = 6,   /* index 0: masked multiview cost of the last aggregated mode (u16, d stride dp) */
    SISTER_DBG_SUM0 = 7,   /* index 0: pass-0 SGM sum of the last aggregated mode (u16, Hp x Wp x dp); needs
                              SISTER_TUNE_FULL_DISP = 1 (otherwise only the original pixels' sums are kept) */
    SISTER_DBG_DISP = 8,   /* index mode: padded winner-take-all disparity (u16, Hp x Wp); needs SISTER_TUNE_FULL_DISP = 1 */
    SISTER_DBG_DP = 9      /* returns the padded disparity stride dp of the volumes in *(int*)dst */
};
SISTER_API int sister_debug_fetch(sister_ctx *ctx, int what, int index, void *host_dst, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
