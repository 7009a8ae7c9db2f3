// TEST INFRASTRUCTURE ONLY. Built by oracle/build_ref.sh into oracle/_ref/ together with the
// reference's own, unmodified stage sources (cpp/src/sister/census.cpp, postprocess.cpp, sgm.cpp).
//
// OpenCV is not available, so the OpenCV glue of cpp/include/sister/SisterMultiviewDisparities.hpp is
// restated here literally (copyMakeBorder, flip, transpose, the mask and masked-sum loops, convertTo,
// ROI crop, *255). The stage functions themselves are the reference's compiled code. Deviation from
// the reference, by necessity: every volume is zero-filled, which pins the Hamming rows the reference
// never writes (census.cpp:123-145) to 0.
#include "stereoalgo.h"

#include <cstdlib>
#include <cstring>
#include <vector>

// defined in census.cpp without a header declaration
void censusTransform(uint8 *source, uint64 *dest, uint32 width, uint32 height, uint8 rw, uint8 rh);

namespace {

template <typename T> T *amalloc(size_t n) {
    T *p = (T *)_mm_malloc(n * sizeof(T) + 64, 64);
    if (p) memset(p, 0, n * sizeof(T) + 64);
    return p;
}

struct Img {  // minimal row-major u8 image
    int rows = 0, cols = 0;
    std::vector<uint8_t> px;
    Img() {}
    Img(int r, int c) : rows(r), cols(c), px((size_t)r * c) {}
    uint8_t &at(int r, int c) { return px[(size_t)r * cols + c]; }
    uint8_t at(int r, int c) const { return px[(size_t)r * cols + c]; }
};

// copyMakeBorder(src, dst, dc, dc, dc, dc, BORDER_REPLICATE)
Img pad_replicate(const uint8_t *src, int w, int h, int dc) {
    Img o(h + 2 * dc, w + 2 * dc);
    for (int r = 0; r < o.rows; r++)
        for (int c = 0; c < o.cols; c++) {
            int y = r - dc, x = c - dc;
            y = y < 0 ? 0 : (y >= h ? h - 1 : y);
            x = x < 0 ? 0 : (x >= w ? w - 1 : x);
            o.at(r, c) = src[(size_t)y * w + x];
        }
    return o;
}
Img transpose(const Img &a) {
    Img o(a.cols, a.rows);
    for (int r = 0; r < a.rows; r++)
        for (int c = 0; c < a.cols; c++) o.at(c, r) = a.at(r, c);
    return o;
}
// cv::flip: code 0 flips rows (vertical), 1 flips columns (horizontal), -1 both
Img flip(const Img &a, int code) {
    Img o(a.rows, a.cols);
    for (int r = 0; r < a.rows; r++)
        for (int c = 0; c < a.cols; c++) {
            int rr = (code == 0 || code == -1) ? a.rows - 1 - r : r;
            int cc = (code == 1 || code == -1) ? a.cols - 1 - c : c;
            o.at(rr, cc) = a.at(r, c);
        }
    return o;
}

// doMultiStereo (hpp:152-295), literal, with the helper-class masks kept as u8 row-major arrays.
void do_multi_stereo(uint8 *imC, uint8 *im0, uint8 *imCto90, uint8 *im90, uint8 *imCto180, uint8 *im180,
                     uint8 *imCto270, uint8 *im270, float32 *outputL, int width, int height, int dispCount,
                     int mode) {
    const int maxDisp = dispCount - 1;
    const size_t plane = (size_t)width * height, vol = plane * dispCount;
    float32 *ptrL_hw = amalloc<float32>(plane), *ptrR_hw = amalloc<float32>(plane);
    float32 *ptrL_wh = amalloc<float32>(plane), *ptrR_wh = amalloc<float32>(plane);
    uint16 *dsiC0 = amalloc<uint16>(vol), *dsiC90 = amalloc<uint16>(vol), *dsiC180 = amalloc<uint16>(vol),
           *dsiC270 = amalloc<uint16>(vol), *dsiC90f = amalloc<uint16>(vol), *dsiC180f = amalloc<uint16>(vol),
           *dsiC270f = amalloc<uint16>(vol), *multidsi = amalloc<uint16>(vol), *sum_dsi = amalloc<uint16>(vol);

    ad_census(imC, im0, height, width, dispCount, dsiC0, 4);
    ad_census(imCto90, im90, width, height, dispCount, dsiC90f, 4);
    ad_census(imCto180, im180, height, width, dispCount, dsiC180f, 4);
    ad_census(imCto270, im270, width, height, dispCount, dsiC270f, 4);

    std::vector<uint8_t> lrc0(plane), lrc90(plane), lrc180(plane), lrc270(plane);
    if (mode != 2) {
        WTALeft_SSE(ptrL_hw, dsiC0, width, height, maxDisp, 1);
        WTARight_SSE(ptrR_hw, dsiC0, width, height, maxDisp, 1);
        median3x3_SSE(ptrL_hw, ptrL_hw, width, height);
        median3x3_SSE(ptrR_hw, ptrR_hw, width, height);
        doLRCheck(ptrL_hw, ptrR_hw, width, height, 5);
        for (int i = 0; i < height; i++)
            for (int j = 0; j < width; j++)
                lrc0[(size_t)i * width + j] = (ptrL_hw[i * width + j] <= 0 || j < dispCount) ? 0 : 1;
        WTALeft_SSE(ptrL_hw, dsiC180f, width, height, maxDisp, 1);
        WTARight_SSE(ptrR_hw, dsiC180f, width, height, maxDisp, 1);
        median3x3_SSE(ptrL_hw, ptrL_hw, width, height);
        median3x3_SSE(ptrR_hw, ptrR_hw, width, height);
        doLRCheck(ptrL_hw, ptrR_hw, width, height, 5);
        for (int i = 0; i < height; i++)
            for (int j = 0; j < width; j++)
                lrc180[(size_t)i * width + (width - 1 - j)] = (ptrL_hw[i * width + j] <= 0 || j < dispCount) ? 0 : 1;
    }
    if (mode != 1) {
        Img m90(width, height), m270(width, height);
        WTALeft_SSE(ptrL_wh, dsiC90f, height, width, maxDisp, 1);
        WTARight_SSE(ptrR_wh, dsiC90f, height, width, maxDisp, 1);
        median3x3_SSE(ptrL_wh, ptrL_wh, height, width);
        median3x3_SSE(ptrR_wh, ptrR_wh, height, width);
        doLRCheck(ptrL_wh, ptrR_wh, height, width, 5);
        for (int i = 0; i < width; i++)
            for (int j = 0; j < height; j++) m90.at(i, j) = (ptrL_wh[i * height + j] <= 0 || j < dispCount) ? 0 : 1;
        Img t = flip(transpose(m90), -1);
        memcpy(lrc90.data(), t.px.data(), plane);
        WTALeft_SSE(ptrL_wh, dsiC270f, height, width, maxDisp, 1);
        WTARight_SSE(ptrR_wh, dsiC270f, height, width, maxDisp, 1);
        median3x3_SSE(ptrL_wh, ptrL_wh, height, width);
        median3x3_SSE(ptrR_wh, ptrR_wh, height, width);
        doLRCheck(ptrL_wh, ptrR_wh, height, width, 5);
        for (int i = 0; i < width; i++)
            for (int j = 0; j < height; j++) m270.at(i, j) = (ptrL_wh[i * height + j] <= 0 || j < dispCount) ? 0 : 1;
        t = flip(transpose(m270), 1);
        memcpy(lrc270.data(), t.px.data(), plane);
    }

    for (int i = 0; i < height; i++)
        for (int j = 0; j < width; j++) {
            const size_t p = (size_t)i * width + j;
            for (int d = 0; d < dispCount; d++) {
                const size_t o = p * dispCount + d;
                dsiC180[o] = dsiC180f[(size_t)i * width * dispCount + (size_t)(width - 1 - j) * dispCount + d];
                dsiC90[o] = dsiC90f[(size_t)(width - 1 - j) * height * dispCount + (size_t)(height - 1 - i) * dispCount + d];
                dsiC270[o] = dsiC270f[(size_t)(width - 1 - j) * height * dispCount + (size_t)i * dispCount + d];
                int v;
                switch (mode) {
                case 0: v = lrc0[p] * dsiC0[o] + lrc180[p] * dsiC180[o] + lrc90[p] * dsiC90[o] + lrc270[p] * dsiC270[o]; break;
                case 1: v = lrc0[p] * dsiC0[o] + lrc180[p] * dsiC180[o]; break;
                default: v = lrc90[p] * dsiC90[o] + lrc270[p] * dsiC270[o]; break;
                }
                multidsi[o] = (uint16)v;
            }
        }

    // sgm reads the center image one byte before and after its rows (sgm.cpp:170, :227-232); the image
    // does not influence the result (alpha = 0), but the reads must stay inside an allocation.
    uint8 *img = amalloc<uint8>(plane + 2 * width + 64);
    memcpy(img + width, imC, plane);
    sgm(img + width, height, width, dispCount, multidsi, sum_dsi, 7, 17, 8);
    WTALeft_SSE(outputL, sum_dsi, width, height, maxDisp, 1);

    _mm_free(img);
    _mm_free(ptrL_hw); _mm_free(ptrR_hw); _mm_free(ptrL_wh); _mm_free(ptrR_wh);
    _mm_free(dsiC0); _mm_free(dsiC90); _mm_free(dsiC180); _mm_free(dsiC270);
    _mm_free(dsiC90f); _mm_free(dsiC180f); _mm_free(dsiC270f); _mm_free(multidsi); _mm_free(sum_dsi);
}

}  // namespace

extern "C" {

void ref_census(const uint8_t *img, int W, int H, uint64_t *out) {
    uint8 *a = amalloc<uint8>((size_t)W * H);
    uint64 *o = amalloc<uint64>((size_t)W * H);
    memcpy(a, img, (size_t)W * H);
    censusTransform(a, o, W, H, 4, 3);
    memcpy(out, o, (size_t)W * H * 8);
    _mm_free(a); _mm_free(o);
}

// ad_census of one frame pair (census.cpp:149-158), H rows x W cols, volume zero-filled first.
void ref_ad_census(const uint8_t *a, const uint8_t *b, int W, int H, int D, uint16_t *vol) {
    const size_t plane = (size_t)W * H;
    uint8 *x = amalloc<uint8>(plane), *y = amalloc<uint8>(plane);
    uint16 *v = amalloc<uint16>(plane * D);
    memcpy(x, a, plane); memcpy(y, b, plane);
    ad_census(x, y, H, W, D, v, 4);
    memcpy(vol, v, plane * D * 2);
    _mm_free(x); _mm_free(y); _mm_free(v);
}

void ref_wta(const uint16_t *vol, int W, int H, int D, int right, float *out) {
    const size_t plane = (size_t)W * H;
    uint16 *v = amalloc<uint16>(plane * D);
    float32 *o = amalloc<float32>(plane);
    memcpy(v, vol, plane * D * 2);
    if (right) WTARight_SSE(o, v, W, H, D - 1, 1);
    else WTALeft_SSE(o, v, W, H, D - 1, 1);
    memcpy(out, o, plane * 4);
    _mm_free(v); _mm_free(o);
}

void ref_median_inplace(float *a, int W, int H) {
    const size_t plane = (size_t)W * H;
    float32 *o = amalloc<float32>(plane);
    memcpy(o, a, plane * 4);
    median3x3_SSE(o, o, W, H);
    memcpy(a, o, plane * 4);
    _mm_free(o);
}

void ref_lrcheck(float *L, const float *R, int W, int H) {
    doLRCheck(L, (float32 *)R, W, H, 5);
}

void ref_sgm(const uint16_t *C, int W, int H, int D, uint16_t *S) {
    const size_t plane = (size_t)W * H;
    uint16 *c = amalloc<uint16>(plane * D), *s = amalloc<uint16>(plane * D);
    uint8 *img = amalloc<uint8>(plane + 2 * W + 64);
    memcpy(c, C, plane * D * 2);
    sgm(img + W, H, W, D, c, s, 7, 17, 8);
    memcpy(S, s, plane * D * 2);
    _mm_free(c); _mm_free(s); _mm_free(img);
}

// compute_disparities (hpp:26-119) on gray views {center, right, top, left, bottom}; any output may be
// NULL (that mode is skipped). Requires dc <= 256 (WTARight_SSE's store[256+32], postprocess.cpp:193).
int ref_compute(const uint8_t *const views[5], int w, int h, int dc, uint16_t *out_multi, uint16_t *out_h,
                uint16_t *out_v) {
    if (dc < 8 || dc > 256 || dc % 8 || w % 4 || h % 4) return 1;
    Img imC = pad_replicate(views[0], w, h, dc), im0 = pad_replicate(views[1], w, h, dc),
        im90 = pad_replicate(views[2], w, h, dc), im180 = pad_replicate(views[3], w, h, dc),
        im270 = pad_replicate(views[4], w, h, dc);
    const int width = imC.cols, height = imC.rows;
    Img imCf_to180 = flip(imC, 1), im180f = flip(im180, 1);
    Img imCf_to90 = flip(transpose(imC), -1), im90f = flip(transpose(im90), -1);
    Img imCf_to270 = flip(transpose(imC), 0), im270f = flip(transpose(im270), 0);
    uint16_t *outs[3] = {out_multi, out_h, out_v};
    float32 *disp = amalloc<float32>((size_t)width * height);
    for (int mode = 0; mode < 3; mode++) {
        if (!outs[mode]) continue;
        do_multi_stereo(imC.px.data(), im0.px.data(), imCf_to90.px.data(), im90f.px.data(), imCf_to180.px.data(),
                        im180f.px.data(), imCf_to270.px.data(), im270f.px.data(), disp, width, height, dc, mode);
        for (int i = 0; i < h; i++)
            for (int j = 0; j < w; j++) {
                // convertTo(CV_16UC1) rounds (values are integral), then *255 saturating
                float f = disp[(size_t)(i + dc) * width + (j + dc)];
                unsigned u = f <= 0 ? 0u : (unsigned)(f + 0.5f);
                unsigned s = u * 255u;
                outs[mode][(size_t)i * w + j] = (uint16_t)(s > 65535u ? 65535u : s);
            }
    }
    _mm_free(disp);
    return 0;
}

}  // extern "C"
