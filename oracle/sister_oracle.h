/*
 * Oracle for the SiSter 5-view disparity path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain, portable C restatement of the reference CPU algorithm
 * (cpp/include/sister/SisterMultiviewDisparities.hpp + cpp/src/sister/{census,postprocess,sgm}.cpp).
 * It is the checker for the CUDA path: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it. The product library never links it.
 *
 * Parity pin: every stage is cross-checked against the reference's own stage code compiled
 * from its sources (oracle/_ref, built by oracle/build_ref.sh where the reference tree and an
 * x86 compiler are present), and the end-to-end outputs against golden fixtures produced by
 * that compiled reference (tests/golden/).
 *
 * Geometry (all images row-major):
 *   w, h        original view size; dc = dispCount ("max disparity"), D = dc disparities 0..dc-1
 *   Wp = w+2dc, Hp = h+2dc   replicate-padded size
 *   frame f in {0: 0deg (center vs right), 1: 90deg (center vs top), 2: 180deg (center vs left),
 *               3: 270deg (center vs bottom)}; frames 0/2 are Hp rows x Wp cols, frames 1/3 are
 *               Wp rows x Hp cols.
 *   Cost / sum volumes are [row][col][d], d fastest.
 */
#ifndef SISTER_ORACLE_H
#define SISTER_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Eight frame images, frame f's center image first, then its neighbour:
 * out + (2f)*Wp*Hp = center frame f, out + (2f+1)*Wp*Hp = neighbour frame f.
 * views[5] = {center, right, top, left, bottom} (reference ctor order), w x h gray u8, tightly packed. */
void orc_frames(const uint8_t *const views[5], int w, int h, int dc, uint8_t *out);

/* 9x7 census with the reference's carry-over bit 63 (census.cpp:30-51). */
void orc_census(const uint8_t *img, int W, int H, uint64_t *out);

/* Full Hamming volume exactly as hammingCost stores it (census.cpp:54-146), unwritten rows = 0. */
void orc_cost_volume(const uint64_t *cc, const uint64_t *cn, int W, int H, int D, uint16_t *vol);

/* WTA-left / WTA-right of a pair's Hamming volume, computed from census words (postprocess.cpp:74-315). */
void orc_wta_lr(const uint64_t *cc, const uint64_t *cn, int W, int H, int D, uint16_t *L, uint16_t *R);

/* In-place 3x3 median with the reference's flattened, row-recursive semantics (postprocess.cpp:15-71). */
void orc_median_inplace(uint16_t *a, int W, int H);

/* LR check + confidence mask in frame coordinates (postprocess.cpp:318-341, hpp:201-251). */
void orc_lrc_mask(const uint16_t *L, const uint16_t *R, int W, int H, int dc, uint8_t *mask);

/* Frame mask -> original padded coordinates (hpp:216, :235-236, :250-251). */
void orc_mask_to_orig(const uint8_t *mask_frame, int f, int Wp, int Hp, uint8_t *mask_orig);

/* Masked multiview cost for a mode (hpp:255-277): mode 0 all four pairs, 1 horizontal, 2 vertical. */
void orc_masked_cost(const uint64_t *const census[8], const uint8_t *const masks[4], int Wp, int Hp,
                     int D, int mode, uint16_t *M);

/* 8-path SGM, P1=7, P2=100, two passes with the reference's first-line semantics (sgm.cpp:26-455). */
void orc_sgm(const uint16_t *C, int W, int H, int D, uint16_t *S);
/* The same, stopping after `npasses` (1: pass 0 only, leaving the pass-0 sum in S). */
void orc_sgm_passes(const uint16_t *C, int W, int H, int D, uint16_t *S, int npasses);

/* WTA-left (argmin over d<=min(j,D-1), lowest d on ties) of a volume. */
void orc_wta_left_vol(const uint16_t *vol, int W, int H, int D, uint16_t *disp);
void orc_wta_right_vol(const uint16_t *vol, int W, int H, int D, uint16_t *disp);
void orc_lrcheck(const uint16_t *L, const uint16_t *R, int W, int H, int16_t *out);
int orc_stereo(const uint8_t *center, const uint8_t *other, int w, int h, int D, int16_t *L_out, uint16_t *R_out);

/* Crop [dc,dc+h)x[dc,dc+w) and scale by 255 with u16 saturation (hpp:111-118). */
void orc_crop_scale(const uint16_t *disp, int Wp, int dc, int w, int h, uint16_t *out);

/* Whole compute_disparities (hpp:26-119). Any of out_multi / out_h / out_v may be NULL; the mode is
 * then skipped. Returns 0 on success, nonzero on invalid arguments or allocation failure.
 * If masks_out != NULL it receives the four original-coordinate masks (4*Wp*Hp bytes). */
int orc_compute(const uint8_t *const views[5], int w, int h, int dc, uint16_t *out_multi, uint16_t *out_h,
                uint16_t *out_v, uint8_t *masks_out);

/* One mode of compute_disparities in bounded host memory (the masked cost recomputed row by row, only the
 * pass-0 sum volume stored, the final WTA taken as pass 1 completes each row): same results as orc_compute,
 * for rigs too large to hold the cost and sum volumes together. mode 0 multiview, 1 horizontal, 2 vertical;
 * out = w*h (disparity*255), disp_padded = Hp*Wp padded disparity or NULL. Returns 0, 1 (bad arguments) or 2
 * (out of memory). */
int orc_compute_stream(const uint8_t *const views[5], int w, int h, int dc, int mode, uint16_t *out,
                       uint16_t *disp_padded);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int orc_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
