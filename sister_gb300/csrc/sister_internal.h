// Internal declarations shared by the sm_103a kernels and the host runtime of libsister_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <vector>

namespace sister {

// Geometry of one rig (reference naming: width/height are the padded frame sizes of doMultiStereo,
// SisterMultiviewDisparities.hpp:41).
struct Geom {
    int w, h;     // original view size
    int dc;       // dispCount; disparities 0..dc-1
    int Wp, Hp;   // replicate-padded size w+2dc, h+2dc
    int dp;       // d-stride of the cost/sum volumes: dc rounded up to 32*dpl, padding holds 0xFFFF
    int dpl;      // disparities per lane in the aggregation kernels (dp / 32)
    size_t plane; // Wp*Hp
    __host__ __device__ int frows(int f) const { return (f & 1) ? Wp : Hp; }
    __host__ __device__ int fcols(int f) const { return (f & 1) ? Hp : Wp; }
};

// Lanes per pixel are fixed at 32; dpl is chosen from this list (the smallest >= ceil(dc/32)); every
// choice is even so that a lane's slice of a volume row is 4-byte aligned.
constexpr int kDplChoices[] = {2, 4, 6, 8, 12, 16};
int choose_dpl(int dc);
Geom make_geom(int w, int h, int dc);

// Band hand-off progress counters sit one per 128-byte line: the next band polls its counter from another SM
// while the writer updates it, and neighbouring bands' counters must not share the line.
constexpr int kProgressStride = 32;
inline size_t progress_bytes(size_t ncounters) { return ncounters * kProgressStride * sizeof(unsigned); }
// progress counters of an aggregation launch with `nitems` work items, plus one more line for the launch's item
// ticket (the counter CTAs draw their next work item from)
inline size_t sgm_progress_bytes(size_t nitems) { return progress_bytes(nitems + 1); }

// Device-side error codes written by kernels with bounded waits.
enum : unsigned { kErrNone = 0, kErrTimeout = 1 };
// Default limit of a device-side wait on another warp or CTA (microseconds); a context may lower it
// (SISTER_TUNE_WAIT_LIMIT_US). Waits for a warp's own asynchronous copies in flight (before its barriers are
// reused or the CTA exits) always use kDrainLimitUs: those copies complete by themselves within microseconds,
// and they must have landed before the shared memory they write is reused.
constexpr unsigned kDefaultWaitUs = 2000000;
constexpr unsigned kDrainLimitUs = 2000000;

// One rig's aggregation buffers (all device pointers).
struct SgmRig {
    const uint16_t *cost; // [Hp][Wp][dp] masked multiview cost
    uint16_t *sum0;       // [sh][sw][dp] 4-path sum of pass 0 (top-down) over the stored window
    uint16_t *sum1;       // [sh][sw][dp] 4-path sum of pass 1 (bottom-up) over the stored window
    uint16_t *bnd;        // [2][2][Wp][3dp+8] r1/r2/r3 states + minima of a band's last row: pass, band parity
    unsigned *progress;   // [2][nbands] x kProgressStride: pixels of a band's last row published so far, per
                          // pass, one counter per 128-byte line (zeroed first)
    int W, H, D;          // padded width and height, max disparity dc
    int nbands;           // bands per pass = ceil(H / R)
    // Window of padded pixels whose sums are stored: columns [sx0, sx0 + sw), rows [sy0, sy0 + sh). sw = 0 stores
    // the whole padded plane; sgm_crop_window keeps only the original image (the only pixels the final WTA reads
    // when no padded map is asked for).
    int sx0, sy0, sw, sh;
    // [sh][sw] disparity*255 (saturated): when set (with a cropped window), the launch also runs the final WTA of
    // every output row as work items after the band items; else the sums are left for launch_sgm_wta
    uint16_t *out;
};
// Store only the original image's pixels (padded offset dc) of the pass sums: volumes of w*h*dp cells.
inline void sgm_crop_window(SgmRig &r, const Geom &g) {
    r.sx0 = g.dc;
    r.sy0 = g.dc;
    r.sw = g.w;
    r.sh = g.h;
}
// cells of one pass-sum volume: the original image with a cropped window, else the padded plane
inline size_t sgm_sum_cells(const Geom &g, bool cropped) { return (cropped ? (size_t)g.w * g.h : g.plane) * g.dp; }

// Work items of a multi-rig aggregation launch: rig << 24 | kind | index << 1 | pass. A band item (index = band)
// aggregates R rows of one pass; a fused final-WTA item (kind kItemWta, index = a row of the original image) takes
// the winner-take-all of one output row once both passes' bands holding it are done. All band items of a launch
// come before its WTA items.
constexpr uint32_t kItemWta = 1u << 23, kItemIndexMask = (1u << 22) - 1u;
inline uint32_t sgm_item_band(int rig, int band, int pass) { return (uint32_t)rig << 24 | (uint32_t)band << 1 | (uint32_t)pass; }
inline uint32_t sgm_item_wta(int rig, int row) { return (uint32_t)rig << 24 | kItemWta | (uint32_t)row << 1; }
// The j-th output row in WTA item order: the rows nearest the middle of the image first (both passes finish the
// middle bands first), then alternately one above and one below.
__host__ __device__ inline int sgm_wta_row(int j, int h) { return h / 2 + ((j & 1) ? -((j + 1) >> 1) : (j >> 1)); }

// Arguments of one aggregation launch: the work items of one or several rigs that share the d-stride dp
// (same kernel instantiation) and the band height R.
struct SgmLaunch {
    SgmRig rig0;            // the rig of a single-rig launch (rigs == nullptr): item k = pass k & 1, band k >> 1
    const SgmRig *rigs;     // device array of rigs (multi-rig launch), or nullptr
    const uint32_t *items;  // device array, rig << 24 | band << 1 | pass, in an order where every item comes
                            // after the previous band of its rig and pass (multi-rig launch), or nullptr
    int nitems;
    int R, dp;              // rows per band (one warp per row + fetcher and writer per CTA); d-stride
    unsigned *claim;        // item ticket, zero at launch: a CTA takes its next work item from an atomic add
    unsigned *err;          // device error flag
    unsigned wait_limit_us; // longest wait of any warp (microseconds) before reporting kErrTimeout
};

// Launch plan of the aggregation kernel for one geometry.
struct SgmPlan {
    int R = 0, cs = 0, nbands = 0, ngroups = 0, nclusters = 0;
};

// one-time per-device kernel attribute setup (dynamic shared memory limits)
void init_mask_kernels();
void init_sgm_kernels();
void init_cost_kernels(); // shared-memory limit of the cost kernels on this device

// ---- kernel launchers (all asynchronous on `st`) ----
// views_dev: 5 planes of w*h gray bytes, tightly packed, order {center, right, top, left, bottom}
void launch_to_gray(const uint8_t *const src[5], int stride, int channels, int w, int h, uint8_t *views_dev,
                    cudaStream_t st);
void launch_frames(const uint8_t *views_dev, const Geom &g, uint8_t *frames, cudaStream_t st);
// census of the first nimg frame images (8: all four frame pairs; 2: frame 0 only)
void launch_census(const uint8_t *frames, const Geom &g, uint64_t *census, cudaStream_t st, int nimg = 8);
// the mask stages run on frames [f0, f0 + nf) (all four by default)
// rowflags (4 x max(Wp, Hp) u32, or null): pair WTA publishes each frame row with `epoch`; a median given the
// same flags waits for the rows it reads, so it may be launched before the frame's pair WTA has finished.

// the medians' row-flag waits use the default limit (kDefaultWaitUs)
void launch_median(const uint16_t *wta, const Geom &g, uint16_t *med, cudaStream_t st, int f0 = 0, int nf = 4,
                   const unsigned *rowflags = nullptr, unsigned epoch = 0, unsigned *err = nullptr);
// pair WTA of every frame and the eight medians in one launch (medians follow the rows through rowflags)
void launch_wta_median(const uint64_t *census, const Geom &g, uint16_t *wta, uint16_t *med, unsigned *rowflags,
                       unsigned epoch, unsigned *err, cudaStream_t st);
// two-view doStereo tail: LR-checked left map (-10 where rejected) and the right map, from frame 0's medians
void launch_stereo_lrc(const uint16_t *med, const Geom &g, int16_t *outL, uint16_t *outR, cudaStream_t st);
void launch_lrc_mask(const uint16_t *med, const Geom &g, uint8_t *masks, cudaStream_t st, int f0 = 0, int nf = 4);
void launch_masked_cost(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                        cudaStream_t st);
// Aggregation: both passes in one persistent launch (sums into sum0 / sum1), then the final WTA, crop and
// *255 over the sum of the two. Return cudaError_t.
// force_R: 0 = choose automatically; force_cs is accepted and ignored (groups are single bands)
SgmPlan sgm_plan(const Geom &g, int device, int force_R = 0, int force_cs = 0);
SgmPlan sgm_plan_gb300(const Geom &g); // the plan on a 152-SM GB300, without a device query
// band hand-off records of one rig: two rows of Wp records per pass, reused by every other band (independent of
// the plan)
size_t sgm_bnd_bytes(const Geom &g, const SgmPlan &p);
// single rig: rig.nbands is filled from the plan; rig.progress (sgm_progress_bytes(p.ngroups): the counters and
// the item ticket) is zeroed here; with rig.out set the launch also takes the final WTA (rig.sh more items)
cudaError_t launch_sgm(const Geom &g, const SgmPlan &p, SgmRig rig, unsigned *err, cudaStream_t st,
                       unsigned wait_limit_us = kDefaultWaitUs);
// several rigs of one d-stride class: rigs / items in device memory (progress counters and the item ticket
// `claim` already zeroed); grid = min(nitems, resident CTAs)
int sgm_rows_max(int dp, int device);
int sgm_rows_gb300(int dp); // sgm_rows_max on a GB300, without a device query
cudaError_t launch_sgm_multi(int dp, int R, const SgmRig *rigs_dev, const uint32_t *items_dev, int nitems,
                             unsigned *claim, unsigned *err, int device, cudaStream_t st,
                             unsigned wait_limit_us = kDefaultWaitUs);
// Work items of a multi-rig launch. Band items are ordered by band (then rig, then pass), so every item follows the
// previous band of its rig and pass. With `fuse`, every rig's output rows (rows sy0 .. sy0+sh-1 of its padded
// plane) follow all band items as final-WTA items, in the order in which their two bands come in the band order
// (nearest the middle first among equals). Spreading them among the band items instead (each one grid of items
// after its bands) measured slower: a CTA drawn away from the bands lengthens the wavefront's critical path.
// rigs: {nbands, H, sy0, sh}.
struct SgmItemRig {
    int nbands, H, sy0, sh;
};
void sgm_build_items(const SgmItemRig *rigs, int nrigs, int R, bool fuse, std::vector<uint32_t> &items);
// out: [h][w] disparity*255, disp: [Hp][Wp] padded disparity; either may be null
// WTARight over S0 + S1 (two-view doStereo): lowest k <= min(dc-1, Wp-1-b) minimising S(i, b+k, k)
cudaError_t launch_sgm_wta_right(const Geom &g, const uint16_t *s0, const uint16_t *s1, uint16_t *disp,
                                 cudaStream_t st);
// disp (padded Hp x Wp map) may be null: then only the cropped output pixels are computed. cropped: the sums hold
// only the original image's pixels (sgm_crop_window; disp must then be null)
cudaError_t launch_sgm_wta(const Geom &g, const uint16_t *sum0, const uint16_t *sum1, uint16_t *out, uint16_t *disp,
                           cudaStream_t st, bool cropped);

} // namespace sister
