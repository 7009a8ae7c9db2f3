// Internal declarations shared by the sm_103a kernels and the host runtime of libsister_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

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

// Device-side error codes written by kernels with bounded waits.
enum : unsigned { kErrNone = 0, kErrTimeout = 1 };

// Per-launch arguments of the aggregation (SGM) kernel.
struct SgmArgs {
    const uint16_t *cost; // [Hp][Wp][dp] masked multiview cost
    uint16_t *sum0;       // [Hp][Wp][dp] pass-0 path sum (written by pass 0, read by pass 1)
    uint16_t *bnd;        // [nbands][Wp][3dp+8] r1/r2/r3 states + minima of each band's last row
    unsigned *progress;   // [nbands] pixels of a band's last row published so far
    unsigned *err;        // device error flag
    uint16_t *out;        // [h][w] disparity*255 (pass 1), may be null
    uint16_t *disp;       // [Hp][Wp] padded WTA disparity (pass 1), may be null
    int W, H, D, dp, dc, w, h;
    int R;                // rows per band (4 path warps per row + fetcher + publisher per CTA)
    int cs;               // bands per group: always 1 (bands are not clustered)
    int nbands, ngroups;
    unsigned wait_limit_us; // longest wait of any warp (microseconds) before reporting kErrTimeout
};

// Launch plan of the aggregation kernel for one geometry.
struct SgmPlan {
    int R = 0, cs = 0, nbands = 0, ngroups = 0, nclusters = 0;
};

// one-time per-device kernel attribute setup (dynamic shared memory limits)
void init_mask_kernels();
void init_sgm_kernels();

// ---- kernel launchers (all asynchronous on `st`) ----
// views_dev: 5 planes of w*h gray bytes, tightly packed, order {center, right, top, left, bottom}
void launch_to_gray(const uint8_t *const src[5], int stride, int channels, int w, int h, uint8_t *views_dev,
                    cudaStream_t st);
void launch_frames(const uint8_t *views_dev, const Geom &g, uint8_t *frames, cudaStream_t st);
void launch_census(const uint8_t *frames, const Geom &g, uint64_t *census, cudaStream_t st);
void launch_pair_wta(const uint64_t *census, const Geom &g, uint16_t *wta, cudaStream_t st);
void launch_median(const uint16_t *wta, const Geom &g, uint16_t *med, cudaStream_t st);
void launch_lrc_mask(const uint16_t *med, const Geom &g, uint8_t *masks, cudaStream_t st);
void launch_masked_cost(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                        cudaStream_t st);
// Both aggregation passes plus the final WTA, crop and *255. Returns a cudaError_t.
// force_R: 0 = choose automatically; force_cs is accepted and ignored (groups are single bands)
SgmPlan sgm_plan(const Geom &g, int device, int force_R = 0, int force_cs = 0);
size_t sgm_bnd_bytes(const Geom &g, const SgmPlan &p);
// one aggregation pass (0: top-down, stores the pass sum; 1: bottom-up, adds it and reduces)
cudaError_t launch_sgm_pass(const Geom &g, const SgmPlan &p, SgmArgs a, int pass, cudaStream_t st);

} // namespace sister
