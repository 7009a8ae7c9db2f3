"""Regenerate the golden fixtures from the reference's own compiled code (oracle/_ref).

Run from the repository root on an x86-64 host that has the reference tree, passing its path:
    python tests/golden/make_golden.py --reference PATH [--c2] [--stereo-only]
    python tests/golden/make_golden.py --c5

Every case stores the SHA-256 of its five input views (so a test first checks that the seeded
generator reproduces the same bytes on the machine it runs on) and the reference outputs of the three
modes of compute_disparities. Small cases also store the inputs themselves.

--c5 writes the stress rig's fixture (4096x3000, max disparity 512, mode 0). The reference cannot run that rig
(its nine full volumes take 190 GB and its WTARight_SSE overflows a stack buffer above 256 disparities,
postprocess.cpp:193), so this fixture comes from the oracle's bounded-memory restatement
(orc_compute_stream), which the other fixtures pin: it reproduces every reference-made fixture here bit for
bit (tests/test_oracle.py). Needs about 24 GB of host memory and a few minutes.
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from sister_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def views_sha(views) -> str:
    h = hashlib.sha256()
    for v in views:
        h.update(np.ascontiguousarray(v, np.uint8).tobytes())
    return h.hexdigest()


def out_sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.uint16).tobytes()).hexdigest()


def small_cases():
    """(name, views, dc) for the small fixtures: random-texture and synthetic-scene rigs."""
    rng = np.random.default_rng(20240901)
    cases = []
    for (h, w, dc) in [(16, 24, 8), (32, 40, 16), (24, 64, 24)]:
        cases.append(("rand_%dx%d_dc%d" % (w, h, dc), [rng.integers(0, 256, (h, w), dtype=np.uint8) for _ in range(5)], dc))
    for k, (w, h, dc) in enumerate([(64, 48, 16), (96, 64, 24), (128, 96, 40), (160, 120, 64), (200, 148, 72),
                                   (96, 200, 32)]):
        dmax = max(dc - 8, 6)
        views, _ = synth.make_rig(w, h, 2, dmax, seed=100 + k, tiles=4)
        cases.append(("synth_%dx%d_dc%d" % (w, h, dc), views, dc))
    return cases


def stereo_cases():
    """(name, center, other, dc) for the two-view doStereo fixtures: random pairs and synthetic center/right pairs."""
    rng = np.random.default_rng(20241203)
    cases = []
    for (h, w, dc) in [(16, 24, 8), (32, 48, 16)]:
        cases.append(("stereo_rand_%dx%d_dc%d" % (w, h, dc), rng.integers(0, 256, (h, w), dtype=np.uint8),
                      rng.integers(0, 256, (h, w), dtype=np.uint8), dc))
    for k, (w, h, dc) in enumerate([(96, 64, 24), (160, 120, 48), (200, 148, 64)]):
        views, _ = synth.make_rig(w, h, 2, dc - 8, seed=300 + k, tiles=4)
        cases.append(("stereo_synth_%dx%d_dc%d" % (w, h, dc), views[0], views[1], dc))
    return cases


def make_stereo(ref):
    for name, center, other, dc in stereo_cases():
        L, R = ref.stereo(center, other, dc)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), center=center, other=other, dc=dc,
                            left=L.astype(np.int16), right=R.astype(np.uint16))
        print(name)


def make_c5():
    """The stress rig's fixture from the bounded-memory oracle (see the module docstring)."""
    t0 = time.time()
    (views, _), dc = synth.rig_c5(5)
    port = oracle.Port()
    out, pad = port.compute_stream(views, dc, 0, padded=True)
    h, w = out.shape
    d = pad[dc:dc + h, dc:dc + w]
    assert np.array_equal(out, np.minimum(d.astype(np.int64) * 255, 65535).astype(np.uint16))
    np.savez_compressed(os.path.join(HERE, "c5_4096x3000_dc512.npz"), dc=dc, seed=5, views_sha=views_sha(views),
                        multi_sha=out_sha(out), multi_d=d.astype(np.uint16),
                        source="oracle orc_compute_stream (mode 0), %d OpenMP threads" % port.num_threads())
    print("c5 %.1fs" % (time.time() - t0))


def main():
    if "--c5" in sys.argv:
        make_c5()
        return
    if "--reference" not in sys.argv:
        sys.exit("pass --reference PATH (the reference project tree) or --c5")
    os.environ["SISTER_REFERENCE"] = sys.argv[sys.argv.index("--reference") + 1]
    ref = oracle.Ref()
    t0 = time.time()
    make_stereo(ref)
    if "--stereo-only" in sys.argv:
        return
    for name, views, dc in small_cases():
        multi, horiz, vert = ref.compute(views, dc)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), views=np.stack(views), dc=dc, multi=multi,
                            horiz=horiz, vert=vert, views_sha=views_sha(views))
        print("%-24s %.2fs" % (name, time.time() - t0))
    (views, gt), dc = synth.rig_c1(1)
    multi, horiz, vert = ref.compute(views, dc)
    np.savez_compressed(os.path.join(HERE, "c1_640x480_dc192.npz"), dc=dc, seed=1, views_sha=views_sha(views),
                        multi_sha=out_sha(multi), horiz_sha=out_sha(horiz), vert_sha=out_sha(vert),
                        multi_d=(multi // 255).astype(np.uint8), horiz_d=(horiz // 255).astype(np.uint8),
                        vert_d=(vert // 255).astype(np.uint8))
    print("c1 %.2fs" % (time.time() - t0))
    if "--c2" in sys.argv:
        (views, gt), dc = synth.rig_c2(2)
        multi, horiz, vert = ref.compute(views, dc)
        np.savez_compressed(os.path.join(HERE, "c2_1920x1080_dc256.npz"), dc=dc, seed=2, views_sha=views_sha(views),
                            multi_sha=out_sha(multi), horiz_sha=out_sha(horiz), vert_sha=out_sha(vert),
                            multi_d=(multi // 255).astype(np.uint8))
        print("c2 %.2fs" % (time.time() - t0))


if __name__ == "__main__":
    main()
