// sister_gb300.hpp -- header-only C++ mirror of the reference helper class over the C ABI
// (include/sister_gb300.h). Drop-in for cpp/include/sister/SisterMultiviewDisparities.hpp:18-119:
//
//   sister::MultiviewDisparities m(center, right, top, left, bottom);     // hpp:22
//   m.compute_disparities(dispCount, multi, horiz, vert);                 // hpp:26
//
// Images are plain views (pointer, size, pitch, channels) so the header needs no OpenCV; define
// SISTER_WITH_OPENCV before including it to get cv::Mat overloads with the reference's exact signatures.
// Outputs are u16 images of the input size holding disparity*255, bit-exact with the reference.
#pragma once

#include "sister_gb300.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef SISTER_WITH_OPENCV
#include <opencv2/core.hpp>
#endif

namespace sister {

struct ImageView {
    const uint8_t *data = nullptr;
    int width = 0, height = 0;
    int stride = 0;   // bytes per row
    int channels = 1; // 1 = gray, 3 = BGR
};

struct Image16 {
    std::vector<uint16_t> pixels; // row-major, width*height
    int width = 0, height = 0;
};

class Error : public std::runtime_error {
  public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

  private:
    int code_;
};

class MultiviewDisparities {
  public:
    MultiviewDisparities(ImageView center, ImageView right, ImageView top, ImageView left, ImageView bottom,
                         int device = 0)
        : views_{center, right, top, left, bottom} {
        if (sister_ctx_create(&ctx_, device) != SISTER_OK) throw Error(SISTER_EDEVICE, "sister_ctx_create failed");
        const uint8_t *p[5];
        for (int k = 0; k < 5; k++) {
            if (views_[k].width != center.width || views_[k].height != center.height ||
                views_[k].channels != center.channels)
                throw Error(SISTER_EINVAL, "all five views must have the same size and channel count");
            p[k] = views_[k].data;
        }
        check(sister_load_views(ctx_, p, center.width, center.height, center.stride, center.channels));
    }
    ~MultiviewDisparities() { sister_ctx_destroy(ctx_); }
    MultiviewDisparities(const MultiviewDisparities &) = delete;
    MultiviewDisparities &operator=(const MultiviewDisparities &) = delete;

    // compute_disparities (hpp:26): the three modes of the reference; pass nullptr to skip a mode.
    void compute_disparities(int dispCount, Image16 *disp_multiview, Image16 *disp_horizontal, Image16 *disp_vertical) {
        check(sister_set_max_disparity(ctx_, dispCount));
        Image16 *outs[3] = {disp_multiview, disp_horizontal, disp_vertical};
        uint16_t *ptr[3] = {nullptr, nullptr, nullptr};
        for (int m = 0; m < 3; m++) {
            if (!outs[m]) continue;
            outs[m]->width = views_[0].width;
            outs[m]->height = views_[0].height;
            outs[m]->pixels.resize((size_t)views_[0].width * views_[0].height);
            ptr[m] = outs[m]->pixels.data();
        }
        check(sister_compute(ctx_, ptr[0], ptr[1], ptr[2]));
    }

#ifdef SISTER_WITH_OPENCV
    MultiviewDisparities(cv::Mat center, cv::Mat right, cv::Mat top, cv::Mat left, cv::Mat bottom, int device = 0)
        : MultiviewDisparities(view(center), view(right), view(top), view(left), view(bottom), device) {
        keep_ = {center, right, top, left, bottom};
    }
    void compute_disparities(int dispCount, cv::Mat &disp_multiview, cv::Mat &disp_horizontal, cv::Mat &disp_vertical) {
        const int h = views_[0].height, w = views_[0].width;
        disp_multiview.create(h, w, CV_16UC1);
        disp_horizontal.create(h, w, CV_16UC1);
        disp_vertical.create(h, w, CV_16UC1);
        check(sister_set_max_disparity(ctx_, dispCount));
        check(sister_compute(ctx_, disp_multiview.ptr<uint16_t>(), disp_horizontal.ptr<uint16_t>(),
                             disp_vertical.ptr<uint16_t>()));
    }
    static ImageView view(const cv::Mat &m) {
        if (m.depth() != CV_8U || !m.isContinuous()) throw Error(SISTER_EINVAL, "expected continuous 8-bit images");
        return ImageView{m.ptr<uint8_t>(), m.cols, m.rows, (int)m.step, m.channels()};
    }
#endif

    sister_ctx *context() { return ctx_; }

  private:
    void check(int rc) {
        if (rc != SISTER_OK) throw Error(rc, sister_last_error(ctx_));
    }
    ImageView views_[5];
    sister_ctx *ctx_ = nullptr;
#ifdef SISTER_WITH_OPENCV
    std::vector<cv::Mat> keep_;
#endif
};

} // namespace sister

// The reference's class name at global scope (SisterMultiviewDisparities.hpp:18), so callers written against the
// reference -- compute_disp.cpp:26-35 constructs `SisterMultiviewDisparities multiview(center, right, top, left,
// bottom)` -- compile unchanged once this header replaces the reference's include.
using SisterMultiviewDisparities = sister::MultiviewDisparities;
