import glob
import hashlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: CPU test of more than a few seconds")


@pytest.fixture(scope="session")
def port():
    import oracle

    return oracle.Port()


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in-tree if needed. No fallback: a missing build is an error."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu test collected on a host without a CUDA device")
    from sister_gb300 import build, load_library

    build.build()
    return load_library()


def views_sha(views) -> str:
    h = hashlib.sha256()
    for v in views:
        h.update(np.ascontiguousarray(v, np.uint8).tobytes())
    return h.hexdigest()


def out_sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.uint16).tobytes()).hexdigest()


def small_golden_files():
    return sorted(f for f in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if os.path.basename(f).startswith(("rand_", "synth_")))


def load_small(path):
    z = np.load(path)
    views = [z["views"][k] for k in range(5)]
    return views, int(z["dc"]), (z["multi"], z["horiz"], z["vert"]), str(z["views_sha"])
