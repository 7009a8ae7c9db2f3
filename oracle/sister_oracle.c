/*
 * Oracle for the SiSter 5-view disparity path -- TEST INFRASTRUCTURE ONLY (see sister_oracle.h).
 *
 * Portable C (no SIMD intrinsics), optional OpenMP over independent rows. Every function cites the
 * reference lines it restates; paths are relative to the reference project root.
 */
#include "sister_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define INF16 65535u

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static inline uint16_t adds16(uint32_t a, uint32_t b) {
    uint32_t s = a + b;
    return s > INF16 ? (uint16_t)INF16 : (uint16_t)s;
}
static inline uint16_t subs16(uint32_t a, uint32_t b) { return a > b ? (uint16_t)(a - b) : 0; }
static inline uint16_t min16(uint16_t a, uint16_t b) { return a < b ? a : b; }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Replicate pad by dc on all sides (hpp:35-39, copyMakeBorder BORDER_REPLICATE) and the four frame
 * orientations (hpp:54-70): f0 identity, f2 = flip(.,1), f1 = flip(transpose(.),-1),
 * f3 = flip(transpose(.),0). Neighbour of frame f: right, top, left, bottom (ctor order hpp:22,
 * doMultiStereo argument order hpp:77). */
void orc_frames(const uint8_t *const views[5], int w, int h, int dc, uint8_t *out) {
    const int Wp = w + 2 * dc, Hp = h + 2 * dc;
    const size_t plane = (size_t)Wp * Hp;
    static const int nb[4] = {1, 2, 3, 4};
    for (int f = 0; f < 4; f++) {
        for (int k = 0; k < 2; k++) {
            const uint8_t *src = views[k == 0 ? 0 : nb[f]];
            uint8_t *dst = out + (size_t)(2 * f + k) * plane;
            const int rows = (f & 1) ? Wp : Hp, cols = (f & 1) ? Hp : Wp;
#pragma omp parallel for schedule(static)
            for (int a = 0; a < rows; a++) {
                for (int b = 0; b < cols; b++) {
                    int y, x;
                    switch (f) {
                    case 0: y = a; x = b; break;
                    case 1: y = Hp - 1 - b; x = Wp - 1 - a; break;
                    case 2: y = a; x = Wp - 1 - b; break;
                    default: y = b; x = Wp - 1 - a; break;
                    }
                    dst[(size_t)a * cols + b] =
                        src[(size_t)clampi(y - dc, 0, h - 1) * w + clampi(x - dc, 0, w - 1)];
                }
            }
        }
    }
}

/* 63 tests of census.cpp:30-35,46-48: bit = I(i+y, j+x) > I(i-y, j-x), y=-3..3 outer, x=-4..4 inner,
 * shifted in from the right. */
static inline uint64_t census63(const uint8_t *img, int W, int i, int j) {
    uint64_t v = 0;
    for (int y = -3; y <= 3; y++)
        for (int x = -4; x <= 4; x++)
            v = (v << 1) | (uint64_t)(img[(size_t)(i + y) * W + (j + x)] > img[(size_t)(i - y) * W + (j - x)]);
    return v;
}

/* censusTransform, census.cpp:38-51. The accumulator is never reset between pixels (:42), so after 63
 * shifts bit 63 holds bit 0 of the previous interior pixel in raster order, i.e. its last test
 * (y=+3, x=+4); the first interior pixel (3,4) gets 0. Non-interior pixels are 0 (:40). */
void orc_census(const uint8_t *img, int W, int H, uint64_t *out) {
    memset(out, 0, (size_t)W * H * sizeof(uint64_t));
#pragma omp parallel for schedule(static)
    for (int i = 3; i < H - 3; i++) {
        for (int j = 4; j < W - 4; j++) {
            uint64_t carry = 0;
            if (!(i == 3 && j == 4)) {
                const int pi = (j > 4) ? i : i - 1, pj = (j > 4) ? j - 1 : W - 5;
                carry = img[(size_t)(pi + 3) * W + pj + 4] > img[(size_t)(pi - 3) * W + pj - 4];
            }
            out[(size_t)i * W + j] = census63(img, W, i, j) | (carry << 63);
        }
    }
}

/* One cell of the pair volume as hammingCost leaves it (census.cpp:54-146): rows 0..2 are 255
 * (written before and again after the OMP sections, :95-98, :142-145); rows H-2, H-1 are never
 * written (the sections cover [2, H-2), :123-135) and are defined here as 0; elsewhere
 * 255 for d > j (:74-78) and popcount(Cc[i][j] ^ Cn[i][j-d]) otherwise (:79-85). */
static inline uint16_t pair_cost(const uint64_t *cc, const uint64_t *cn, int W, int H, int i, int j, int d) {
    if (i < 3) return 255;
    if (i >= H - 2) return 0;
    if (d > j) return 255;
    return (uint16_t)__builtin_popcountll(cc[(size_t)i * W + j] ^ cn[(size_t)i * W + j - d]);
}

void orc_cost_volume(const uint64_t *cc, const uint64_t *cn, int W, int H, int D, uint16_t *vol) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++)
            for (int d = 0; d < D; d++) vol[((size_t)i * W + j) * D + d] = pair_cost(cc, cn, W, H, i, j, d);
}

/* WTALeft_SSE / WTARight_SSE with uniqueness 1.0 (postprocess.cpp:74-185, :187-315). With
 * factorUniq = 1024 the uniqueness test `1024*min <= 1024*secMin` always holds, so both reduce to
 * the first (lowest-index) argmin: left over d in [0, min(j, D-1)] of C(i,j,d); right over
 * k in [0, min(D-1, W-1-j)] of C(i,j+k,k). The reference's -10 branch is unreachable. */
void orc_wta_lr(const uint64_t *cc, const uint64_t *cn, int W, int H, int D, uint16_t *L, uint16_t *R) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            const size_t p = (size_t)i * W + j;
            if (i < 3 || i >= H - 2) { /* constant rows: every cost equal, argmin 0 */
                L[p] = 0;
                R[p] = 0;
                continue;
            }
            int end = j < D - 1 ? j : D - 1, best = 0;
            uint16_t bc = pair_cost(cc, cn, W, H, i, j, 0);
            for (int d = 1; d <= end; d++) {
                const uint16_t c = pair_cost(cc, cn, W, H, i, j, d);
                if (c < bc) { bc = c; best = d; }
            }
            L[p] = (uint16_t)best;
            end = (W - 1 - j) < D - 1 ? W - 1 - j : D - 1;
            best = 0;
            bc = pair_cost(cc, cn, W, H, i, j, 0);
            for (int k = 1; k <= end; k++) {
                const uint16_t c = pair_cost(cc, cn, W, H, i, j + k, k);
                if (c < bc) { bc = c; best = k; }
            }
            R[p] = (uint16_t)best;
        }
    }
}

static inline uint16_t med9(uint16_t *v) {
    /* insertion sort of 9, median = 5th smallest; exact for integer data */
    for (int a = 1; a < 9; a++) {
        uint16_t t = v[a];
        int b = a - 1;
        while (b >= 0 && v[b] > t) { v[b + 1] = v[b]; b--; }
        v[b + 1] = t;
    }
    return v[4];
}

/* median3x3_SSE(src, dst, W, H) called with src == dst (hpp:198-199, 210-211, 226-227, 241-242),
 * postprocess.cpp:15-71. Over the flattened array of N = W*H values:
 *  - x < W: unchanged; x == W: 0 (first store of lastMedian = 0, :29,:61-62; the closing memcpy
 *    :69 is a no-op in place);
 *  - W < x < N-W-4: median of out[x-W-1 .. x-W+1] (already filtered, written earlier in the same
 *    sweep) and in[x-1 .. x+1], in[x+W-1 .. x+W+1] (not yet written); row ends wrap;
 *  - x >= N-W-4: unchanged (the loop stops at :67; the memcpy :70 is a no-op in place). */
void orc_median_inplace(uint16_t *a, int W, int H) {
    const size_t N = (size_t)W * H, Wz = (size_t)W;
    uint16_t *in = (uint16_t *)malloc(N * sizeof(uint16_t));
    if (!in) return;
    memcpy(in, a, N * sizeof(uint16_t));
    a[Wz] = 0;
    for (size_t x = Wz + 1; x + Wz + 4 < N; x++) {
        uint16_t v[9] = {a[x - Wz - 1], a[x - Wz], a[x - Wz + 1], in[x - 1],     in[x],
                         in[x + 1],     in[x + Wz - 1], in[x + Wz], in[x + Wz + 1]};
        a[x] = med9(v);
    }
    free(in);
}

/* doLRCheck(L, R, W, H, 5) (postprocess.cpp:318-341) followed by the confidence mask of
 * hpp:201-206: L' = L if 0 <= L <= j and |L - R[j-L]| <= 5, else -10; mask = (L' > 0 && j >= dc). */
void orc_lrc_mask(const uint16_t *L, const uint16_t *R, int W, int H, int dc, uint8_t *mask) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            const size_t p = (size_t)i * W + j;
            const int base = L[p];
            int v = -10;
            if (base <= j) {
                const int match = R[(size_t)i * W + (j - base)];
                const int diff = base - match;
                if (!(diff > 5 || diff < -5)) v = base;
            }
            mask[p] = (uint8_t)((v > 0 && j >= dc) ? 1 : 0);
        }
    }
}

/* Frame masks back to padded original coordinates: lrc180(i, Wp-1-j) (hpp:216),
 * lrc90 = flip(transpose(.), -1) (hpp:235-236), lrc270 = flip(transpose(.), 1) (hpp:250-251). */
void orc_mask_to_orig(const uint8_t *mf, int f, int Wp, int Hp, uint8_t *mo) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Hp; i++) {
        for (int j = 0; j < Wp; j++) {
            uint8_t v;
            switch (f) {
            case 0: v = mf[(size_t)i * Wp + j]; break;
            case 2: v = mf[(size_t)i * Wp + (Wp - 1 - j)]; break;
            case 1: v = mf[(size_t)(Wp - 1 - j) * Hp + (Hp - 1 - i)]; break;
            default: v = mf[(size_t)(Wp - 1 - j) * Hp + i]; break;
            }
            mo[(size_t)i * Wp + j] = v;
        }
    }
}

/* Pair cost of frame f seen from padded original pixel (i, j) -- the un-rotation of hpp:259-261. */
static inline uint16_t frame_cost(const uint64_t *const census[8], int f, int Wp, int Hp, int i, int j, int d) {
    const uint64_t *cc = census[2 * f], *cn = census[2 * f + 1];
    switch (f) {
    case 0: return pair_cost(cc, cn, Wp, Hp, i, j, d);
    case 2: return pair_cost(cc, cn, Wp, Hp, i, Wp - 1 - j, d);
    case 1: return pair_cost(cc, cn, Hp, Wp, Wp - 1 - j, Hp - 1 - i, d);
    default: return pair_cost(cc, cn, Hp, Wp, Wp - 1 - j, i, d);
    }
}

/* hpp:255-277: multidsi = lrc0*C0 + lrc180*C180 + lrc90*C90 + lrc270*C270 (mode 0), the first two
 * terms (mode 1) or the last two (mode 2). masks[f] is frame f's mask in original coordinates. */
void orc_masked_cost(const uint64_t *const census[8], const uint8_t *const masks[4], int Wp, int Hp, int D,
                     int mode, uint16_t *M) {
    const int use[4] = {mode != 2, mode != 1, mode != 2, mode != 1};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < Hp; i++) {
        for (int j = 0; j < Wp; j++) {
            const size_t p = (size_t)i * Wp + j;
            int m[4];
            for (int f = 0; f < 4; f++) m[f] = use[f] ? masks[f][p] : 0;
            uint16_t *out = M + p * D;
            for (int d = 0; d < D; d++) {
                uint32_t s = 0;
                for (int f = 0; f < 4; f++)
                    if (m[f]) s += frame_cost(census, f, Wp, Hp, i, j, d);
                out[d] = (uint16_t)s;
            }
        }
    }
}

/* 8-path SGM of sgm.cpp:26-455 (called as sgm(.., 7, 17, 8) at hpp:280). P1 = 7; with alpha = 0 and
 * gamma = 100, adaptP2 (:15-22) is the constant 100, so the image never matters.
 * State arrays hold D+2 entries: slot 0 is d = -1 and slot D+1 is d = D, both fixed at 65535
 * (:84-87, :202-206). Column-indexed states carry one 65535 guard column on each side (j = -1 and
 * j = W) whose minimum is 0 (:57-81).
 *  Pass 0 runs rows top-down, columns left-to-right; pass 1 bottom-up, right-to-left (:92-100).
 *  First line of a pass (:103-207): C' = (C == 255 ? 0 : C). The states of paths r1..r3 are set to C'
 *    with minimum min(C'); path r0 starts at the first pixel as C' and then follows the recurrence in
 *    int32 with the result truncated to 8 bits by saturate_cast<uint16>(uint8) (types.h:28, :176);
 *    the sum receives r0 alone (= C' at the first pixel), assigned in pass 0, added mod 2^16 in pass 1.
 *  Remaining lines (:213-440): every path r in {0 (i,j-dj), 1 (i-di,j-dj), 2 (i-di,j), 3 (i-di,j+dj)}
 *    L_r(d) = C(d) +s ( min(Lp(d), Lp(d-1) +s 7, Lp(d+1) +s 7, minLp +s 100) -s minLp ) with u16
 *    saturating +s/-s; r0 restarts each row from Lp = 0, minLp = 0 (:215-216). The sum is
 *    ((r0 +s r1) +s r2) +s r3, stored in pass 0 and added saturating in pass 1 (:386-391). */
void orc_sgm_passes(const uint16_t *C, int W, int H, int D, uint16_t *S, int npasses) {
    const int P = D + 2;
    const size_t colsz = (size_t)(W + 2) * P;
    uint16_t *r1last = (uint16_t *)malloc(colsz * 2), *r1cur = (uint16_t *)malloc(colsz * 2);
    uint16_t *r2 = (uint16_t *)malloc(colsz * 2), *r3 = (uint16_t *)malloc(colsz * 2);
    uint16_t *m1last = (uint16_t *)calloc(W + 2, 2), *m1cur = (uint16_t *)calloc(W + 2, 2);
    uint16_t *m2 = (uint16_t *)calloc(W + 2, 2), *m3 = (uint16_t *)calloc(W + 2, 2);
    uint16_t *r0prev = (uint16_t *)malloc(P * 2), *r0new = (uint16_t *)malloc(P * 2);
    uint16_t *t2 = (uint16_t *)malloc(P * 2), *t3 = (uint16_t *)malloc(P * 2);
    if (!r1last || !r1cur || !r2 || !r3 || !m1last || !m1cur || !m2 || !m3 || !r0prev || !r0new || !t2 || !t3)
        goto out;
    for (size_t k = 0; k < colsz; k++) r1last[k] = r1cur[k] = r2[k] = r3[k] = INF16;
    for (int k = 0; k < P; k++) r0prev[k] = r0new[k] = t2[k] = t3[k] = INF16;

#define ST(arr, c, d) (arr)[(size_t)((c) + 1) * P + (d) + 1]
    for (int pass = 0; pass < npasses; pass++) {
        const int di = pass ? -1 : 1, dj = di;
        const int i1 = pass ? H - 1 : 0, j1 = pass ? W - 1 : 0;
        const int iend = pass ? -1 : H, jend = pass ? -1 : W;

        /* ---- first line ---- */
        {
            const uint16_t *c = C + ((size_t)i1 * W + j1) * D;
            uint16_t *s = S + ((size_t)i1 * W + j1) * D;
            uint16_t mn = INF16;
            for (int d = 0; d < D; d++) {
                const uint16_t v = c[d] == 255 ? 0 : c[d];
                r0prev[d + 1] = v;
                ST(r1last, j1, d) = v;
                ST(r2, j1, d) = v;
                ST(r3, j1, d) = v;
                if (v < mn) mn = v;
                s[d] = pass ? (uint16_t)(s[d] + v) : v;
            }
            uint16_t r0min = mn;
            m1last[j1 + 1] = m2[j1 + 1] = m3[j1 + 1] = mn;
            for (int j = j1 + dj; j != jend; j += dj) {
                c = C + ((size_t)i1 * W + j) * D;
                s = S + ((size_t)i1 * W + j) * D;
                uint16_t mnc = INF16, mn0 = INF16;
                for (int d = 0; d < D; d++) {
                    const uint16_t v = c[d] == 255 ? 0 : c[d];
                    ST(r1last, j, d) = v;
                    ST(r2, j, d) = v;
                    ST(r3, j, d) = v;
                    if (v < mnc) mnc = v;
                    int32_t prop = r0prev[d + 1];
                    int32_t t = (int32_t)r0prev[d] + 7;
                    if (prop > t) prop = t;
                    t = (int32_t)r0prev[d + 2] + 7;
                    if (prop > t) prop = t;
                    t = (int32_t)r0min + 100;
                    if (prop > t) prop = t;
                    prop -= r0min;
                    const uint16_t nv = (uint16_t)(uint8_t)((int32_t)v + prop);
                    r0new[d + 1] = nv;
                    if (nv < mn0) mn0 = nv;
                    s[d] = pass ? (uint16_t)(s[d] + nv) : nv;
                }
                m1last[j + 1] = m2[j + 1] = m3[j + 1] = mnc;
                uint16_t *tmp = r0prev; r0prev = r0new; r0new = tmp;
                r0min = mn0;
            }
        }

        /* ---- remaining lines ---- */
        for (int i = i1 + di; i != iend; i += di) {
            for (int d = 0; d < D; d++) r0prev[d + 1] = 0;
            uint16_t r0min = 0;
            for (int j = j1; j != jend; j += dj) {
                const uint16_t *c = C + ((size_t)i * W + j) * D;
                uint16_t *s = S + ((size_t)i * W + j) * D;
                const uint16_t *p1 = &ST(r1last, j - dj, -1), *p2 = &ST(r2, j, -1), *p3 = &ST(r3, j + dj, -1);
                const uint16_t mp1 = m1last[j - dj + 1], mp2 = m2[j + 1], mp3 = m3[j + dj + 1];
                const uint16_t q0 = adds16(100, r0min), q1 = adds16(100, mp1), q2 = adds16(100, mp2),
                               q3 = adds16(100, mp3);
                uint16_t *n1 = &ST(r1cur, j, -1);
                uint16_t mn0 = INF16, mn1 = INF16, mn2 = INF16, mn3 = INF16;
                for (int d = 1; d <= D; d++) {
                    const uint16_t cd = c[d - 1];
                    const uint16_t v0 = adds16(
                        cd, subs16(min16(min16(r0prev[d], min16(adds16(r0prev[d - 1], 7), adds16(r0prev[d + 1], 7))), q0),
                                   r0min));
                    const uint16_t v1 =
                        adds16(cd, subs16(min16(min16(p1[d], min16(adds16(p1[d - 1], 7), adds16(p1[d + 1], 7))), q1), mp1));
                    const uint16_t v2 =
                        adds16(cd, subs16(min16(min16(p2[d], min16(adds16(p2[d - 1], 7), adds16(p2[d + 1], 7))), q2), mp2));
                    const uint16_t v3 =
                        adds16(cd, subs16(min16(min16(p3[d], min16(adds16(p3[d - 1], 7), adds16(p3[d + 1], 7))), q3), mp3));
                    r0new[d] = v0;
                    n1[d] = v1;
                    t2[d] = v2;
                    t3[d] = v3;
                    if (v0 < mn0) mn0 = v0;
                    if (v1 < mn1) mn1 = v1;
                    if (v2 < mn2) mn2 = v2;
                    if (v3 < mn3) mn3 = v3;
                    const uint16_t ges = adds16(adds16(adds16(v0, v1), v2), v3);
                    s[d - 1] = pass ? adds16(s[d - 1], ges) : ges;
                }
                uint16_t *tmp = r0prev; r0prev = r0new; r0new = tmp;
                r0min = mn0;
                memcpy(&ST(r2, j, 0), &t2[1], (size_t)D * 2);
                memcpy(&ST(r3, j, 0), &t3[1], (size_t)D * 2);
                m1cur[j + 1] = mn1;
                m2[j + 1] = mn2;
                m3[j + 1] = mn3;
            }
            uint16_t *tmp = r1last; r1last = r1cur; r1cur = tmp;
            tmp = m1last; m1last = m1cur; m1cur = tmp;
        }
    }
#undef ST
out:
    free(r1last); free(r1cur); free(r2); free(r3);
    free(m1last); free(m1cur); free(m2); free(m3);
    free(r0prev); free(r0new); free(t2); free(t3);
}

void orc_sgm(const uint16_t *C, int W, int H, int D, uint16_t *S) { orc_sgm_passes(C, W, H, D, S, 2); }

/* Final WTALeft_SSE(outputL, sum_dsi, Wp, Hp, dc-1, 1) (hpp:283): first argmin over d <= min(j, D-1). */
void orc_wta_left_vol(const uint16_t *vol, int W, int H, int D, uint16_t *disp) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            const uint16_t *c = vol + ((size_t)i * W + j) * D;
            const int end = j < D - 1 ? j : D - 1;
            int best = 0;
            uint16_t bc = c[0];
            for (int d = 1; d <= end; d++)
                if (c[d] < bc) { bc = c[d]; best = d; }
            disp[(size_t)i * W + j] = (uint16_t)best;
        }
    }
}

/* WTARight_SSE(disp, vol, W, H, D-1, 1) (postprocess.cpp:187-315): R(j) = the lowest k <= min(D-1, W-1-j)
   minimising vol(i, j+k, k). Both of its branches keep the lowest index (the SSE search replaces the running
   minimum only on a strictly smaller block minimum, _mm_minpos_epu16 returns the lowest index of a block, the
   border loop compares strictly), and uniqueness 1 never rejects (1024 * min <= 1024 * second minimum). */
void orc_wta_right_vol(const uint16_t *vol, int W, int H, int D, uint16_t *disp) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < H; i++) {
        for (int j = 0; j < W; j++) {
            const int end = (W - 1 - j) < (D - 1) ? (W - 1 - j) : (D - 1);
            int best = 0;
            uint16_t bc = vol[((size_t)i * W + j) * D];
            for (int k = 1; k <= end; k++) {
                const uint16_t c = vol[((size_t)i * W + j + k) * D + k];
                if (c < bc) { bc = c; best = k; }
            }
            disp[(size_t)i * W + j] = (uint16_t)best;
        }
    }
}

/* doLRCheck(L, R, W, H, 5) (postprocess.cpp:318-341) on integer maps: L(i, j) is kept where 0 <= L <= j and
   |L - R(i, j - L)| <= 5, else it becomes -10. */
void orc_lrcheck(const uint16_t *L, const uint16_t *R, int W, int H, int16_t *out) {
    for (int i = 0; i < H; i++)
        for (int j = 0; j < W; j++) {
            const int b = L[(size_t)i * W + j];
            int keep = 0;
            if (b <= j) {
                const int diff = b - (int)R[(size_t)i * W + j - b];
                keep = diff <= 5 && diff >= -5;
            }
            out[(size_t)i * W + j] = keep ? (int16_t)b : (int16_t)-10;
        }
}

/* doStereo (SisterMultiviewDisparities.hpp:122-150): ad_census -> sgm -> WTALeft / WTARight -> in-place medians
   -> doLRCheck, on unpadded w x h images. L gets -10 where the LR check rejects; R is the median-filtered right map.
   Returns 0, or -1 when memory runs out. */
int orc_stereo(const uint8_t *center, const uint8_t *other, int w, int h, int D, int16_t *L_out, uint16_t *R_out) {
    const size_t plane = (size_t)w * h;
    uint64_t *cc = (uint64_t *)malloc(plane * 8), *cn = (uint64_t *)malloc(plane * 8);
    uint16_t *vol = (uint16_t *)malloc(plane * D * 2), *S = (uint16_t *)malloc(plane * D * 2);
    uint16_t *L = (uint16_t *)malloc(plane * 2);
    int rc = -1;
    if (cc && cn && vol && S && L) {
        orc_census(center, w, h, cc);
        orc_census(other, w, h, cn);
        orc_cost_volume(cc, cn, w, h, D, vol);
        orc_sgm(vol, w, h, D, S);
        orc_wta_left_vol(S, w, h, D, L);
        orc_wta_right_vol(S, w, h, D, R_out);
        orc_median_inplace(L, w, h);
        orc_median_inplace(R_out, w, h);
        orc_lrcheck(L, R_out, w, h, L_out);
        rc = 0;
    }
    free(cc); free(cn); free(vol); free(S); free(L);
    return rc;
}

/* convertTo(CV_16UC1), ROI Rect(dc, dc, Wp-2dc, Hp-2dc), then * 255 with u16 saturation (hpp:111-118). */
void orc_crop_scale(const uint16_t *disp, int Wp, int dc, int w, int h, uint16_t *out) {
    for (int i = 0; i < h; i++)
        for (int j = 0; j < w; j++) {
            const uint32_t v = (uint32_t)disp[(size_t)(i + dc) * Wp + (j + dc)] * 255u;
            out[(size_t)i * w + j] = v > INF16 ? (uint16_t)INF16 : (uint16_t)v;
        }
}

/* Pre-aggregation stages of compute_disparities (hpp:29-70, :188-252): frames, census and the four confidence
 * masks in padded original coordinates. census: 8 * Wp*Hp words, masks: 4 * Wp*Hp bytes. Returns 0, or 2 when
 * memory runs out. */
static int prep_stages(const uint8_t *const views[5], int w, int h, int dc, uint64_t *census, uint8_t *masks) {
    const int Wp = w + 2 * dc, Hp = h + 2 * dc;
    const size_t plane = (size_t)Wp * Hp;
    uint8_t *frames = (uint8_t *)malloc(8 * plane);
    uint8_t *mframe = (uint8_t *)malloc(plane);
    uint16_t *L = (uint16_t *)malloc(plane * 2), *R = (uint16_t *)malloc(plane * 2);
    int rc = 2;
    if (frames && mframe && L && R) {
        orc_frames(views, w, h, dc, frames);
        for (int k = 0; k < 8; k++) {
            const int f = k / 2, rows = (f & 1) ? Wp : Hp, cols = (f & 1) ? Hp : Wp;
            orc_census(frames + k * plane, cols, rows, census + k * plane);
        }
        for (int f = 0; f < 4; f++) {
            const int rows = (f & 1) ? Wp : Hp, cols = (f & 1) ? Hp : Wp;
            orc_wta_lr(census + (2 * f) * plane, census + (2 * f + 1) * plane, cols, rows, dc, L, R);
            orc_median_inplace(L, cols, rows);
            orc_median_inplace(R, cols, rows);
            orc_lrc_mask(L, R, cols, rows, dc, mframe);
            orc_mask_to_orig(mframe, f, Wp, Hp, masks + f * plane);
        }
        rc = 0;
    }
    free(frames); free(mframe); free(L); free(R);
    return rc;
}

/* One row i of the masked multiview cost (the loop body of hpp:255-277 for a fixed i): Wp * D cells. */
static void masked_cost_row(const uint64_t *const census[8], const uint8_t *const masks[4], int Wp, int Hp, int D,
                            int mode, int i, uint16_t *row) {
    const int use[4] = {mode != 2, mode != 1, mode != 2, mode != 1};
#pragma omp parallel for schedule(static)
    for (int j = 0; j < Wp; j++) {
        const size_t p = (size_t)i * Wp + j;
        int m[4];
        for (int f = 0; f < 4; f++) m[f] = use[f] ? masks[f][p] : 0;
        uint16_t *out = row + (size_t)j * D;
        for (int d = 0; d < D; d++) {
            uint32_t s = 0;
            for (int f = 0; f < 4; f++)
                if (m[f]) s += frame_cost(census, f, Wp, Hp, i, j, d);
            out[d] = (uint16_t)s;
        }
    }
}

/* One remaining-lines path update of sgm.cpp:278-383 for one pixel: L(d) = C(d) +s (min(Lp(d), Lp(d-1) +s 7,
 * Lp(d+1) +s 7, minLp +s 100) -s minLp), Lp with guard slots Lp[-1] = Lp[D] = 65535; returns min L. */
static inline uint16_t path_update(const uint16_t *c, const uint16_t *lp, uint16_t mlp, uint16_t *ln, int D) {
    const uint16_t q = adds16(100, mlp);
    uint16_t mn = INF16;
    for (int d = 1; d <= D; d++) {
        const uint16_t v =
            adds16(c[d - 1], subs16(min16(min16(lp[d], min16(adds16(lp[d - 1], 7), adds16(lp[d + 1], 7))), q), mlp));
        ln[d] = v;
        if (v < mn) mn = v;
    }
    return mn;
}

/* compute_disparities for one mode, restated in bounded memory for rigs whose volumes do not fit twice in host
 * memory (4096x3000 at dc 512: 21.1 GB per u16 volume). Same arithmetic as orc_compute, organised differently:
 *  - the masked cost M (hpp:255-277) is never stored: each pass recomputes row i of M from the census words and
 *    masks when it reaches that row;
 *  - the pass-0 sum is the only volume held (Hp*Wp*dc u16); pass 1 adds to it row by row (sgm.cpp:187, :390)
 *    and, once a row is final, takes its WTALeft (hpp:283) into the padded map at once;
 *  - within a row, path r0 (sgm.cpp:215-297, restarted per row) runs first along the row; r1, r2 and r3 read
 *    only the previous row's states (double-buffered here instead of updated in place), so their pixels are
 *    independent and run in parallel; the per-pixel sum keeps the reference's order ((r0 + r1) + r2) + r3 with
 *    u16 saturation (sgm.cpp:388).
 * The first line of each pass follows sgm.cpp:103-207 exactly as orc_sgm_passes does. out: w*h (crop, *255),
 * disp_padded: Hp*Wp (may be NULL). Returns 0, 1 on bad arguments, 2 when memory runs out. */
int orc_compute_stream(const uint8_t *const views[5], int w, int h, int dc, int mode, uint16_t *out,
                       uint16_t *disp_padded) {
    if (w < 4 || h < 4 || dc < 8 || dc % 8 || w % 4 || h % 4 || mode < 0 || mode > 2 || !out) return 1;
    for (int k = 0; k < 5; k++)
        if (!views[k]) return 1;
    const int Wp = w + 2 * dc, Hp = h + 2 * dc, D = dc, P = D + 2, W = Wp, H = Hp;
    const size_t plane = (size_t)Wp * Hp;
    const size_t colsz = (size_t)(W + 2) * P;
    int rc = 2;
    uint64_t *census = (uint64_t *)malloc(8 * plane * sizeof(uint64_t));
    uint8_t *masks = (uint8_t *)calloc(4 * plane, 1);
    uint16_t *disp = (uint16_t *)malloc(plane * 2);
    uint16_t *S = (uint16_t *)malloc(plane * (size_t)D * 2);
    uint16_t *crow = (uint16_t *)malloc((size_t)W * D * 2);
    uint16_t *r0row = (uint16_t *)malloc((size_t)W * D * 2); /* r0 of every pixel of the row */
    uint16_t *st[6];                                           /* r1, r2, r3 states: last and current row */
    uint16_t *mn[6];
    for (int k = 0; k < 6; k++) {
        st[k] = (uint16_t *)malloc(colsz * 2);
        mn[k] = (uint16_t *)calloc(W + 2, 2);
    }
    uint16_t *r0a = (uint16_t *)malloc(P * 2), *r0b = (uint16_t *)malloc(P * 2);
    int ok = census && masks && disp && S && crow && r0row && r0a && r0b;
    for (int k = 0; k < 6; k++) ok = ok && st[k] && mn[k];
    if (!ok) goto done;
    rc = prep_stages(views, w, h, dc, census, masks);
    if (rc) goto done;
    {
        const uint64_t *cptr[8];
        for (int k = 0; k < 8; k++) cptr[k] = census + k * plane;
        const uint8_t *mptr[4] = {masks, masks + plane, masks + 2 * plane, masks + 3 * plane};
        for (int k = 0; k < 6; k++)
            for (size_t q = 0; q < colsz; q++) st[k][q] = INF16;
        /* st[0..2]: r1, r2, r3 of the previous row; st[3..5]: of the row being computed */
#define ST(arr, c, d) (arr)[(size_t)((c) + 1) * P + (d) + 1]
        for (int pass = 0; pass < 2; pass++) {
            const int di = pass ? -1 : 1, dj = di;
            const int i1 = pass ? H - 1 : 0, j1 = pass ? W - 1 : 0;
            const int iend = pass ? -1 : H, jend = pass ? -1 : W;
            for (int k = 0; k < 6; k++) {
                for (size_t q = 0; q < colsz; q++) st[k][q] = INF16;
                memset(mn[k], 0, (size_t)(W + 2) * 2);
            }
            /* ---- first line (sgm.cpp:103-207) ---- */
            masked_cost_row(cptr, mptr, Wp, Hp, D, mode, i1, crow);
            {
                uint16_t *s = S + (size_t)i1 * W * D;
                uint16_t r0min = 0;
                for (int k = 0; k < P; k++) r0a[k] = r0b[k] = INF16;
                for (int j = j1; j != jend; j += dj) {
                    const uint16_t *c = crow + (size_t)j * D;
                    uint16_t *sj = s + (size_t)j * D;
                    uint16_t mnc = INF16, mn0 = INF16;
                    for (int d = 0; d < D; d++) {
                        const uint16_t v = c[d] == 255 ? 0 : c[d];
                        ST(st[0], j, d) = v;
                        ST(st[1], j, d) = v;
                        ST(st[2], j, d) = v;
                        if (v < mnc) mnc = v;
                        uint16_t nv;
                        if (j == j1) {
                            nv = v;
                        } else {
                            int32_t prop = r0a[d + 1];
                            int32_t t = (int32_t)r0a[d] + 7;
                            if (prop > t) prop = t;
                            t = (int32_t)r0a[d + 2] + 7;
                            if (prop > t) prop = t;
                            t = (int32_t)r0min + 100;
                            if (prop > t) prop = t;
                            prop -= r0min;
                            nv = (uint16_t)(uint8_t)((int32_t)v + prop);
                        }
                        r0b[d + 1] = nv;
                        if (nv < mn0) mn0 = nv;
                        sj[d] = pass ? (uint16_t)(sj[d] + nv) : nv;
                    }
                    mn[0][j + 1] = mn[1][j + 1] = mn[2][j + 1] = mnc;
                    uint16_t *tmp = r0a; r0a = r0b; r0b = tmp;
                    r0min = j == j1 ? mnc : mn0;
                }
            }
            if (pass) {
#pragma omp parallel for schedule(static)
                for (int j = 0; j < W; j++) {
                    const uint16_t *c = S + ((size_t)i1 * W + j) * D;
                    const int end = j < D - 1 ? j : D - 1;
                    int best = 0;
                    for (int d = 1; d <= end; d++)
                        if (c[d] < c[best]) best = d;
                    disp[(size_t)i1 * W + j] = (uint16_t)best;
                }
            }
            /* ---- remaining lines (sgm.cpp:213-440) ---- */
            for (int i = i1 + di; i != iend; i += di) {
                masked_cost_row(cptr, mptr, Wp, Hp, D, mode, i, crow);
                /* r0 along the row: restarts from Lp = 0, minLp = 0 (sgm.cpp:215-216) */
                {
                    for (int k = 0; k < P; k++) r0a[k] = INF16;
                    for (int d = 0; d < D; d++) r0a[d + 1] = 0;
                    uint16_t r0min = 0;
                    for (int j = j1; j != jend; j += dj) {
                        r0b[0] = r0b[D + 1] = INF16;
                        const uint16_t m0 = path_update(crow + (size_t)j * D, r0a, r0min, r0b, D);
                        memcpy(r0row + (size_t)j * D, r0b + 1, (size_t)D * 2);
                        uint16_t *tmp = r0a; r0a = r0b; r0b = tmp;
                        r0min = m0;
                    }
                }
                uint16_t *S_row = S + (size_t)i * W * D;
#pragma omp parallel for schedule(static)
                for (int j = 0; j < W; j++) {
                    uint16_t n1[P], n2[P], n3[P];
                    n1[0] = n2[0] = n3[0] = n1[D + 1] = n2[D + 1] = n3[D + 1] = INF16;
                    const uint16_t *c = crow + (size_t)j * D;
                    const uint16_t m1 = path_update(c, &ST(st[0], j - dj, -1), mn[0][j - dj + 1], n1, D);
                    const uint16_t m2 = path_update(c, &ST(st[1], j, -1), mn[1][j + 1], n2, D);
                    const uint16_t m3 = path_update(c, &ST(st[2], j + dj, -1), mn[2][j + dj + 1], n3, D);
                    const uint16_t *v0 = r0row + (size_t)j * D;
                    uint16_t *s = S_row + (size_t)j * D;
                    for (int d = 0; d < D; d++) {
                        const uint16_t ges = adds16(adds16(adds16(v0[d], n1[d + 1]), n2[d + 1]), n3[d + 1]);
                        s[d] = pass ? adds16(s[d], ges) : ges;
                    }
                    memcpy(&ST(st[3], j, 0), n1 + 1, (size_t)D * 2);
                    memcpy(&ST(st[4], j, 0), n2 + 1, (size_t)D * 2);
                    memcpy(&ST(st[5], j, 0), n3 + 1, (size_t)D * 2);
                    mn[3][j + 1] = m1;
                    mn[4][j + 1] = m2;
                    mn[5][j + 1] = m3;
                    if (pass) { /* the row's sums are final: WTALeft (hpp:283) */
                        const int end = j < D - 1 ? j : D - 1;
                        int best = 0;
                        for (int d = 1; d <= end; d++)
                            if (s[d] < s[best]) best = d;
                        disp[(size_t)i * W + j] = (uint16_t)best;
                    }
                }
                for (int k = 0; k < 3; k++) {
                    uint16_t *t = st[k]; st[k] = st[k + 3]; st[k + 3] = t;
                    t = mn[k]; mn[k] = mn[k + 3]; mn[k + 3] = t;
                }
            }
        }
#undef ST
        orc_crop_scale(disp, Wp, dc, w, h, out);
        if (disp_padded) memcpy(disp_padded, disp, plane * 2);
        rc = 0;
    }
done:
    free(census); free(masks); free(disp); free(S); free(crow); free(r0row); free(r0a); free(r0b);
    for (int k = 0; k < 6; k++) {
        free(st[k]);
        free(mn[k]);
    }
    return rc;
}

int orc_compute(const uint8_t *const views[5], int w, int h, int dc, uint16_t *out_multi, uint16_t *out_h,
                uint16_t *out_v, uint8_t *masks_out) {
    if (w < 4 || h < 4 || dc < 8 || dc % 8 || w % 4 || h % 4) return 1;
    for (int k = 0; k < 5; k++)
        if (!views[k]) return 1;
    const int Wp = w + 2 * dc, Hp = h + 2 * dc;
    const size_t plane = (size_t)Wp * Hp;
    int rc = 2;
    uint8_t *frames = (uint8_t *)malloc(8 * plane);
    uint64_t *census = (uint64_t *)malloc(8 * plane * sizeof(uint64_t));
    uint8_t *masks = (uint8_t *)calloc(4 * plane, 1);
    uint8_t *mframe = (uint8_t *)malloc(plane);
    uint16_t *L = (uint16_t *)malloc(plane * 2), *R = (uint16_t *)malloc(plane * 2);
    uint16_t *disp = (uint16_t *)malloc(plane * 2);
    uint16_t *M = NULL, *S = NULL;
    if (!frames || !census || !masks || !mframe || !L || !R || !disp) goto done;

    orc_frames(views, w, h, dc, frames);
    for (int k = 0; k < 8; k++) {
        const int f = k / 2, rows = (f & 1) ? Wp : Hp, cols = (f & 1) ? Hp : Wp;
        orc_census(frames + k * plane, cols, rows, census + k * plane);
    }
    for (int f = 0; f < 4; f++) {
        const int rows = (f & 1) ? Wp : Hp, cols = (f & 1) ? Hp : Wp;
        orc_wta_lr(census + (2 * f) * plane, census + (2 * f + 1) * plane, cols, rows, dc, L, R);
        orc_median_inplace(L, cols, rows);
        orc_median_inplace(R, cols, rows);
        orc_lrc_mask(L, R, cols, rows, dc, mframe);
        orc_mask_to_orig(mframe, f, Wp, Hp, masks + f * plane);
    }
    if (masks_out) memcpy(masks_out, masks, 4 * plane);

    if (out_multi || out_h || out_v) {
        M = (uint16_t *)malloc(plane * dc * sizeof(uint16_t));
        S = (uint16_t *)malloc(plane * dc * sizeof(uint16_t));
        if (!M || !S) goto done;
        const uint64_t *cptr[8];
        for (int k = 0; k < 8; k++) cptr[k] = census + k * plane;
        const uint8_t *mptr[4] = {masks, masks + plane, masks + 2 * plane, masks + 3 * plane};
        uint16_t *outs[3] = {out_multi, out_h, out_v};
        for (int mode = 0; mode < 3; mode++) {
            if (!outs[mode]) continue;
            orc_masked_cost(cptr, mptr, Wp, Hp, dc, mode, M);
            orc_sgm(M, Wp, Hp, dc, S);
            orc_wta_left_vol(S, Wp, Hp, dc, disp);
            orc_crop_scale(disp, Wp, dc, w, h, outs[mode]);
        }
    }
    rc = 0;
done:
    free(frames); free(census); free(masks); free(mframe); free(L); free(R); free(disp); free(M); free(S);
    return rc;
}
