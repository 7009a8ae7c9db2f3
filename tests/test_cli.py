"""sister_compute_disp, the headless replacement of the reference demo (cpp/src/compute_disp.cpp): its PNG
decoder against streams written by zlib (fixed and dynamic Huffman blocks, every row filter, gray and RGB), and
(on the GPU) the whole tool against the library on the same rig."""
import os
import subprocess

import numpy as np
import pytest

from pngutil import read_png_gray, write_png
from sister_gb300 import build, synth


@pytest.fixture(scope="module")
def cli():
    build.build_cli()
    return build.CLI


def test_cli_selftest(cli):
    r = subprocess.run([cli, "--selftest"], capture_output=True, text=True)
    assert r.returncode == 0 and "selftest ok" in r.stdout


@pytest.mark.parametrize("shape,level", [((37, 53), 1), ((64, 48), 9), ((31, 29, 3), 6), ((50, 70, 3), 0),
                                         ((300, 410), 9), ((120, 200, 3), 3)])
def test_png_decoder_matches_zlib_written_images(cli, tmp_path, shape, level):
    rnd = np.random.default_rng(sum(shape) * 7 + level)
    # smooth + noisy content so the deflater emits both literal runs and matches
    base = (np.arange(int(np.prod(shape))) // 5 % 256).reshape(shape)
    img = ((base + rnd.integers(0, 8, shape)) % 256).astype(np.uint8)
    src, raw = str(tmp_path / "in.png"), str(tmp_path / "out.raw")
    write_png(src, img, level)
    r = subprocess.run([cli, "--decode", src, raw], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    w, h, ch = (int(v) for v in r.stdout.split())
    got = np.fromfile(raw, np.uint8)
    if img.ndim == 2:
        assert (w, h, ch) == (shape[1], shape[0], 1)
        assert np.array_equal(got.reshape(h, w), img)
    else:
        assert (w, h, ch) == (shape[1], shape[0], 3)
        assert np.array_equal(got.reshape(h, w, 3), img[:, :, ::-1])  # B, G, R as OpenCV's imread


def test_cli_reports_missing_inputs(cli, tmp_path):
    r = subprocess.run([cli, str(tmp_path) + "/", "64"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


@pytest.mark.gpu
def test_cli_matches_library(cli, gpu_lib, tmp_path):
    import sister_gb300 as sg

    views, _ = synth.make_rig(160, 120, 4, 40, seed=61, tiles=4)
    names = ["center", "right", "top", "left", "bottom"]
    for n, v in zip(names, views):
        write_png(str(tmp_path / (n + ".png")), v)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([cli, str(tmp_path) + "/", "48", "--out", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ctx = sg.Context(0)
    ctx.load_views(views)
    ctx.set_max_disparity(48)
    want = ctx.compute(True, True, True)
    ctx.close()
    for n, wv in zip(["disp_multiview", "disp_horizontal", "disp_vertical"], want):
        got = read_png_gray(str(out / (n + ".png")))
        assert got.dtype == np.uint16 and np.array_equal(got, wv), n
        norm = read_png_gray(str(out / (n + "_norm.png")))
        lo, hi = int(wv.min()), int(wv.max())
        if hi > lo:
            exp = ((wv.astype(np.int64) - lo) * 510 + (hi - lo)) // (2 * (hi - lo))
            assert np.array_equal(norm.astype(np.int64), exp), n + "_norm"
