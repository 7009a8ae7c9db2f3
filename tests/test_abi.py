"""CPU checks of the C-ABI library: it builds, loads, exports every symbol include/*.h declares, and fails
cleanly (status codes, no crash) where no GPU or bad arguments are involved."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT

from sister_gb300 import build as sbuild
import sister_gb300


def declared_symbols():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names += re.findall(r"^\s*SISTER_API\s+(?:int|void|size_t|const char \*)\s*(sister_\w+)\s*\(", src, re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    sbuild.build()
    return sister_gb300.load_library()


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("sister_ctx_create", "sister_ctx_destroy", "sister_load_views", "sister_set_max_disparity",
              "sister_compute", "sister_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_only_declared_symbols_are_exported():
    out = os.popen("nm -D --defined-only %s" % sister_gb300.LIB_PATH).read()
    exported = set(re.findall(r"\s[TW]\s(sister_\w+)", out))
    assert exported == set(declared_symbols())


def test_null_and_invalid_arguments(lib):
    assert lib.sister_set_max_disparity(None, 64) == -1
    assert lib.sister_compute(None, None, None, None) == -1
    assert lib.sister_ctx_create(None, 0) == -1
    assert lib.sister_last_error(None) == b"null context"


def test_device_bytes_estimate(lib):
    small = lib.sister_device_bytes(640, 480, 192)
    big = lib.sister_device_bytes(1920, 1080, 256)
    assert 0 < small < big
    # the aggregation volumes dominate: the u16 cost volume of (w+2dc)(h+2dc)dc and two pass sums of w*h*dc
    assert big >= 2 * (2432 * 1592 + 2 * 1920 * 1080) * 256
    assert lib.sister_device_bytes(0, 480, 192) == 0


def test_no_gpu_context_creation_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert lib.sister_ctx_create(ctypes.byref(h), 0) == -4  # SISTER_EDEVICE
    with pytest.raises(sister_gb300.SisterError):
        sister_gb300.Context(0)


def test_cpp_header_compiles_and_links(tmp_path):
    """The C++ mirror of the reference helper class builds against the library (no GPU needed to link)."""
    src = tmp_path / "use.cpp"
    src.write_text('''
#include "sister_gb300.hpp"
#include <cstdio>
int main(int argc, char **argv) {
    if (argc < 2) { std::printf("%d\\n", (int)sizeof(sister::MultiviewDisparities)); return 0; }
    std::vector<uint8_t> img(64 * 48, 7);
    sister::ImageView v{img.data(), 64, 48, 64, 1};
    try {
        sister::MultiviewDisparities m(v, v, v, v, v);
        sister::Image16 multi, horiz, vert;
        m.compute_disparities(16, &multi, &horiz, &vert);
    } catch (const sister::Error &e) { std::printf("error %d\\n", e.code()); return 1; }
    return 0;
}
''')
    exe = tmp_path / "use"
    libdir = os.path.dirname(sister_gb300.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include", str(src),
           "-L", libdir, "-lsister_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)]
    import subprocess

    subprocess.check_call(cmd)
    assert subprocess.run([str(exe)], capture_output=True).returncode == 0


FAKE_OPENCV = r"""
// minimal stand-in for the few cv::Mat members include/sister_gb300.hpp uses (OpenCV is not installed here)
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <vector>
#define CV_8U 0
#define CV_16UC1 2
namespace cv {
struct Mat {
    int rows = 0, cols = 0, type_ = CV_8U, ch = 1;
    size_t step = 0;
    std::shared_ptr<std::vector<uint8_t>> buf;
    Mat() = default;
    Mat(int r, int c, int t, int channels = 1) { create(r, c, t); ch = channels; step = (size_t)c * channels; buf->resize(step * r); }
    void create(int r, int c, int t) {
        rows = r; cols = c; type_ = t; ch = 1;
        step = (size_t)c * (t == CV_16UC1 ? 2 : 1);
        buf = std::make_shared<std::vector<uint8_t>>(step * r);
    }
    int depth() const { return type_; }
    int channels() const { return ch; }
    bool isContinuous() const { return true; }
    template <class T> T *ptr() { return reinterpret_cast<T *>(buf->data()); }
    template <class T> const T *ptr() const { return reinterpret_cast<const T *>(buf->data()); }
};
}
"""


def test_reference_caller_compiles_against_cpp_header(tmp_path):
    """The calls of the reference's compute_disp.cpp:26-35 -- the global class name SisterMultiviewDisparities
    constructed from five cv::Mat and compute_disparities(dispCount, multi, horiz, vert) into cv::Mat -- compile
    and link unchanged against include/sister_gb300.hpp with SISTER_WITH_OPENCV (cv::Mat faked: no OpenCV here)."""
    import subprocess

    (tmp_path / "opencv2").mkdir()
    (tmp_path / "opencv2" / "core.hpp").write_text(FAKE_OPENCV)
    src = tmp_path / "caller.cpp"
    src.write_text('''
#define SISTER_WITH_OPENCV
#include "sister_gb300.hpp"
#include <cstdio>
int main(int argc, char **argv) {
    if (argc < 2) return 0;
    cv::Mat center(48, 64, CV_8U, 3), right(48, 64, CV_8U, 3), top(48, 64, CV_8U, 3), left(48, 64, CV_8U, 3),
        bottom(48, 64, CV_8U, 3);
    int dispCount = 16;
    try {
        SisterMultiviewDisparities multiview(center, right, top, left, bottom);
        cv::Mat result_horizontal, result_vertical, result_multiview;
        multiview.compute_disparities(dispCount, result_multiview, result_horizontal, result_vertical);
        std::printf("%d %d\\n", result_multiview.rows, result_multiview.cols);
    } catch (const sister::Error &e) { std::printf("error %d\\n", e.code()); return 1; }
    return 0;
}
''')
    exe = tmp_path / "caller"
    libdir = os.path.dirname(sister_gb300.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-I", str(tmp_path), "-I", os.path.join(ROOT, "include"), str(src),
                           "-L", libdir, "-lsister_gb300", "-Wl,-rpath," + libdir, "-o", str(exe)])
    assert subprocess.run([str(exe)], capture_output=True).returncode == 0
