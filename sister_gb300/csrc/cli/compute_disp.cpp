// sister_compute_disp: headless replacement of the reference demo cpp/src/compute_disp.cpp:7-59.
//
//   sister_compute_disp <input folder> <dmax> [--out <dir>] [--device N] [--modes multi,horiz,vert]
//   sister_compute_disp --selftest
//   sister_compute_disp --decode <in.png> <out.raw>   (decoded pixels, gray or B,G,R interleaved)
//
// Like the reference it reads <folder>center.png, right.png, top.png, left.png, bottom.png (the folder string
// is used as a prefix, as in compute_disp.cpp:19-23; 8-bit gray or colour PNGs, colour converted as
// cvtColor BGR2GRAY does) and computes the three disparity images (compute_disparities, :35). Instead of
// OpenCV windows (:51-56) it writes, into --out (default: the input folder):
//   disp_multiview.png, disp_horizontal.png, disp_vertical.png   16-bit gray: disparity*255, exactly the
//                                                                reference's output Mats
//   disp_*_norm.png                                              8-bit min-max normalised previews (as the
//                                                                reference's cv::normalize NORM_MINMAX, :38-40,
//                                                                rounding halves up; its MAGMA colormap is
//                                                                OpenCV data and is not reproduced)
#include "png_io.h"
#include "sister_gb300.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

int usage() {
    std::fprintf(stderr, "usage: sister_compute_disp <input folder> <dmax> [--out <dir>] [--device N] "
                         "[--modes multi,horiz,vert]\n       sister_compute_disp --selftest\n"
                         "       sister_compute_disp --decode <in.png> <out.raw>\n");
    return 2;
}

// NORM_MINMAX to 0..255: round((v - min) * 255 / (max - min)), all zeros when the image is constant
std::vector<uint8_t> normalise(const std::vector<uint16_t> &v) {
    uint16_t lo = 65535, hi = 0;
    for (uint16_t x : v) {
        lo = x < lo ? x : lo;
        hi = x > hi ? x : hi;
    }
    std::vector<uint8_t> out(v.size(), 0);
    if (hi > lo)
        for (size_t i = 0; i < v.size(); i++) out[i] = (uint8_t)(((uint32_t)(v[i] - lo) * 255u * 2 + (hi - lo)) / (2u * (hi - lo)));
    return out;
}

int selftest() {
    // PNG and zlib round trips through the writer and the reader (compressed streams with fixed and dynamic
    // Huffman blocks are exercised by the package's tests, which write the inputs with a real deflater)
    std::vector<uint16_t> img16(37 * 23);
    for (size_t i = 0; i < img16.size(); i++) img16[i] = (uint16_t)(i * 2654435761u >> 16);
    const std::string p16 = "/tmp/sister_selftest16.png";
    if (!pngio::write_png_gray(p16, 37, 23, 16, img16.data()).empty()) return 1;
    std::vector<uint8_t> text;
    const char *s = "sister sister sister GB300\n";
    for (int k = 0; k < 3; k++) text.insert(text.end(), s, s + std::strlen(s));
    std::vector<uint8_t> back;
    const std::vector<uint8_t> z = pngio::zlib_store(text.data(), text.size());
    if (!pngio::zlib_inflate(z.data(), z.size(), back).empty() || back != text) return 3;
    std::vector<uint8_t> img8(64 * 48);
    for (size_t i = 0; i < img8.size(); i++) img8[i] = (uint8_t)(i * 7 + (i >> 6));
    const std::string p8 = "/tmp/sister_selftest8.png";
    pngio::Image rd;
    if (!pngio::write_png_gray(p8, 64, 48, 8, img8.data()).empty() || !pngio::read_png(p8, rd).empty() ||
        rd.width != 64 || rd.height != 48 || rd.channels != 1 || rd.pixels != img8)
        return 4;
    std::remove(p16.c_str());
    std::remove(p8.c_str());
    std::printf("selftest ok\n");
    return 0;
}

} // namespace

int main(int argc, char **argv) {
    if (argc == 2 && !std::strcmp(argv[1], "--selftest")) return selftest();
    if (argc == 4 && !std::strcmp(argv[1], "--decode")) {
        pngio::Image im;
        const std::string e = pngio::read_png(argv[2], im);
        if (!e.empty()) {
            std::fprintf(stderr, "%s\n", e.c_str());
            return 1;
        }
        FILE *f = std::fopen(argv[3], "wb");
        if (!f || std::fwrite(im.pixels.data(), 1, im.pixels.size(), f) != im.pixels.size()) return 1;
        std::fclose(f);
        std::printf("%d %d %d\n", im.width, im.height, im.channels);
        return 0;
    }
    if (argc < 3) return usage();
    const std::string folder = argv[1];
    const int dc = std::atoi(argv[2]);
    std::string outdir = folder;
    int device = 0;
    bool want[3] = {true, true, true};
    for (int a = 3; a < argc; a++) {
        if (!std::strcmp(argv[a], "--out") && a + 1 < argc) {
            outdir = argv[++a];
            if (!outdir.empty() && outdir.back() != '/') outdir += '/';
        } else if (!std::strcmp(argv[a], "--device") && a + 1 < argc) {
            device = std::atoi(argv[++a]);
        } else if (!std::strcmp(argv[a], "--modes") && a + 1 < argc) {
            const std::string m = argv[++a];
            want[0] = m.find("multi") != std::string::npos;
            want[1] = m.find("horiz") != std::string::npos;
            want[2] = m.find("vert") != std::string::npos;
        } else {
            return usage();
        }
    }
    static const char *names[5] = {"center.png", "right.png", "top.png", "left.png", "bottom.png"};
    pngio::Image im[5];
    for (int k = 0; k < 5; k++) {
        const std::string e = pngio::read_png(folder + names[k], im[k]);
        if (!e.empty()) {
            std::fprintf(stderr, "%s\n", e.c_str());
            return 1;
        }
        if (im[k].width != im[0].width || im[k].height != im[0].height || im[k].channels != im[0].channels) {
            std::fprintf(stderr, "%s: size or channel count differs from center.png\n", names[k]);
            return 1;
        }
    }
    const int w = im[0].width, h = im[0].height, ch = im[0].channels;
    sister_ctx *ctx = nullptr;
    int rc = sister_ctx_create(&ctx, device);
    if (rc != SISTER_OK) {
        std::fprintf(stderr, "sister_ctx_create(device %d) failed (%d)\n", device, rc);
        return 1;
    }
    const uint8_t *views[5];
    for (int k = 0; k < 5; k++) views[k] = im[k].pixels.data();
    std::vector<uint16_t> out[3];
    uint16_t *ptr[3] = {nullptr, nullptr, nullptr};
    for (int m = 0; m < 3; m++)
        if (want[m]) {
            out[m].resize((size_t)w * h);
            ptr[m] = out[m].data();
        }
    rc = sister_load_views(ctx, views, w, h, w * ch, ch);
    if (rc == SISTER_OK) rc = sister_set_max_disparity(ctx, dc);
    if (rc == SISTER_OK) rc = sister_compute(ctx, ptr[0], ptr[1], ptr[2]);
    if (rc != SISTER_OK) {
        std::fprintf(stderr, "%s (%d)\n", sister_last_error(ctx), rc);
        sister_ctx_destroy(ctx);
        return 1;
    }
    sister_ctx_destroy(ctx);
    static const char *outn[3] = {"disp_multiview", "disp_horizontal", "disp_vertical"};
    for (int m = 0; m < 3; m++) {
        if (!want[m]) continue;
        std::string e = pngio::write_png_gray(outdir + outn[m] + ".png", w, h, 16, out[m].data());
        if (e.empty()) {
            const std::vector<uint8_t> n8 = normalise(out[m]);
            e = pngio::write_png_gray(outdir + outn[m] + "_norm.png", w, h, 8, n8.data());
        }
        if (!e.empty()) {
            std::fprintf(stderr, "%s\n", e.c_str());
            return 1;
        }
        std::printf("%s%s.png\n", outdir.c_str(), outn[m]);
    }
    return 0;
}
