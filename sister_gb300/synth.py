"""Seeded synthetic 5-view rigs (center, right, top, left, bottom) with known disparity.

The reference ships no dataset and the SiSter dataset is not available offline, so every workload is
synthetic. A rig is built from a seed as follows:

* disparity map: a background plane plus K planar tiles (nearer tiles win), optionally a smooth
  quadratic bump, each plane with a gradient of at most 0.05 px/px, clamped to [dmin, dmax];
* center texture: uniform noise blurred by a separable integer Gaussian (sigma 1.5 or 0.8), stretched
  to 0..255;
* neighbours are the center forward-warped along the direction the matcher searches: at disparity d
  the center pixel (y, x) is compared with right (y, x-d), left (y, x+d), top (y+d, x) and bottom
  (y-d, x); collisions keep the larger disparity (nearer surface); occlusion holes get fresh blurred
  noise;
* every view then receives i.i.d. noise of sigma 2 (Irwin-Hall of 12 uniforms), rounded and clamped
  to u8.

All arithmetic is integer (a splitmix64 counter hash supplies the randomness), so the same seed gives
the same bytes on every platform and numpy version.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)

# integer Gaussian taps round(4096 * exp(-x^2 / (2 sigma^2))) for |x| <= ceil(3 sigma), fixed here so
# that exp() is never evaluated at run time
_KERNELS = {
    1.5: (16, 117, 554, 1684, 3280, 4096, 3280, 1684, 554, 117, 16),
    0.8: (4, 180, 1875, 4096, 1875, 180, 4),
}


def _gauss_kernel(sigma: float) -> np.ndarray:
    if sigma not in _KERNELS:
        raise ValueError("unsupported blur sigma %r" % sigma)
    return np.array(_KERNELS[sigma], np.int64)


def _splitmix(seed: int, stream: int, n: int) -> np.ndarray:
    """n pseudo-random uint64 from a counter-based splitmix64 hash of (seed, stream, index)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03) & 0xFFFFFFFFFFFFFFFF)
        z = base + np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


class _Rand:
    def __init__(self, seed: int):
        self.seed = int(seed) & 0xFFFFFFFF
        self.stream = 0

    def u64(self, n: int) -> np.ndarray:
        self.stream += 1
        return _splitmix(self.seed, self.stream, n)

    def ints(self, lo: int, hi: int, n: int) -> np.ndarray:
        """n integers uniform in [lo, hi] (inclusive)."""
        span = np.uint64(hi - lo + 1)
        return (self.u64(n) % span).astype(np.int64) + lo

    def int1(self, lo: int, hi: int) -> int:
        return int(self.ints(lo, hi, 1)[0])


def _blur(img: np.ndarray, sigma: float) -> np.ndarray:
    k = _gauss_kernel(sigma)
    r = len(k) // 2
    s = int(k.sum())
    a = img.astype(np.int64)
    p = np.pad(a, ((0, 0), (r, r)), mode="edge")
    h = sum(int(k[t]) * p[:, t:t + a.shape[1]] for t in range(len(k)))
    h = (h + s // 2) // s
    p = np.pad(h, ((r, r), (0, 0)), mode="edge")
    v = sum(int(k[t]) * p[t:t + a.shape[0], :] for t in range(len(k)))
    return (v + s // 2) // s


def _texture(rnd: _Rand, h: int, w: int, sigma: float) -> np.ndarray:
    noise = rnd.ints(0, 255, h * w).reshape(h, w)
    b = _blur(noise, sigma)
    lo, hi = int(b.min()), int(b.max())
    return ((b - lo) * 255 // max(hi - lo, 1)).astype(np.int64)


def _plane(rnd: _Rand, h: int, w: int, dmin: int, dmax: int, ys: np.ndarray, xs: np.ndarray) -> np.ndarray:
    """Fixed-point plane d0 + gx*(x-cx) + gy*(y-cy), |gx|,|gy| <= 0.05 px/px, in 1/65536 px."""
    d0 = rnd.int1(dmin, dmax)
    gx = rnd.int1(-3276, 3276)  # 0.05 * 65536
    gy = rnd.int1(-3276, 3276)
    cx, cy = rnd.int1(0, w - 1), rnd.int1(0, h - 1)
    return d0 * 65536 + gx * (xs - cx) + gy * (ys - cy)


def disparity_map(rnd: _Rand, h: int, w: int, dmin: int, dmax: int, tiles: int, bump: bool) -> np.ndarray:
    ys, xs = np.mgrid[0:h, 0:w].astype(np.int64)
    fx = _plane(rnd, h, w, dmin, (dmin + dmax) // 2, ys, xs)  # background: farther half of the range
    for _ in range(tiles):
        tw = rnd.int1(max(w // 12, 4), max(w // 3, 5))
        th = rnd.int1(max(h // 12, 4), max(h // 3, 5))
        x0 = rnd.int1(0, max(w - tw, 0))
        y0 = rnd.int1(0, max(h - th, 0))
        p = _plane(rnd, h, w, dmin, dmax, ys, xs)
        sl = (slice(y0, y0 + th), slice(x0, x0 + tw))
        fx[sl] = np.maximum(fx[sl], p[sl])  # nearer surface wins
    if bump:
        cx, cy = rnd.int1(w // 4, 3 * w // 4), rnd.int1(h // 4, 3 * h // 4)
        rad = rnd.int1(min(h, w) // 6, min(h, w) // 3)
        amp = rnd.int1(5, 30)
        r2 = (xs - cx) ** 2 + (ys - cy) ** 2
        inside = r2 < rad * rad
        fx[inside] += amp * 65536 * (rad * rad - r2[inside]) // (rad * rad)
    d = (fx + 32768) >> 16
    return np.clip(d, dmin, dmax).astype(np.int64)


def _warp(center: np.ndarray, disp: np.ndarray, fill: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """Forward-warp: out(y + dy*d, x + dx*d) = center(y, x); larger d wins collisions; holes <- fill."""
    h, w = center.shape
    ys, xs = np.mgrid[0:h, 0:w]
    ty = ys + dy * disp
    tx = xs + dx * disp
    ok = (ty >= 0) & (ty < h) & (tx >= 0) & (tx < w)
    tidx = (ty * w + tx)[ok]
    dsrc = disp[ok]
    best = np.full(h * w, -1, np.int64)
    np.maximum.at(best, tidx, dsrc)
    win = dsrc == best[tidx]
    out = fill.reshape(-1).copy()
    out[tidx[win]] = center[ok][win]
    return out.reshape(h, w)


def _sensor_noise(rnd: _Rand, img: np.ndarray, sigma2x: int = 2) -> np.ndarray:
    """Add Irwin-Hall(12) noise of std sigma (= sigma2x), round, clamp to u8."""
    n = img.size
    acc = np.zeros(n, np.int64)
    for _ in range(12):
        acc += rnd.ints(0, 65535, n)
    noise = (acc - 12 * 32768) * sigma2x  # ~ N(0, sigma^2) in 1/65536 units
    v = img.reshape(-1) * 65536 + noise
    v = (v + 32768) >> 16
    return np.clip(v, 0, 255).astype(np.uint8).reshape(img.shape)


def make_rig(w: int, h: int, dmin: int, dmax: int, seed: int, tiles: int = 10, bump: bool = False,
             sigma_blur: float = 1.5, native: bool = True):
    """Returns (views, disparity): views = [center, right, top, left, bottom] u8 h x w; disparity int.

    Uses the library's C port of this generator (sister_synth_rig, byte-identical) when the library is
    built and `native` is true, else the numpy definition below (native=False never loads the library)."""
    if native:
        r = _make_rig_native(w, h, dmin, dmax, seed, tiles, bump, sigma_blur)
        if r is not None:
            return r
    return make_rig_numpy(w, h, dmin, dmax, seed, tiles, bump, sigma_blur)


def _make_rig_native(w, h, dmin, dmax, seed, tiles, bump, sigma_blur):
    try:
        from sister_gb300 import load_library
        lib = load_library()
    except (ImportError, OSError):
        return None
    views = np.empty((5, h, w), np.uint8)
    disp = np.empty((h, w), np.int32)
    import ctypes
    f = lib.sister_synth_rig
    f.argtypes = [ctypes.c_int] * 4 + [ctypes.c_longlong, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p]
    rc = f(w, h, dmin, dmax, seed, tiles, int(bool(bump)), int(round(sigma_blur * 10)), views.ctypes.data,
           disp.ctypes.data)
    if rc != 0:
        raise ValueError("sister_synth_rig rejected (%d, %d, %d, %d, %r)" % (w, h, dmin, dmax, sigma_blur))
    return [views[k].copy() for k in range(5)], disp.astype(np.int64)


def make_rig_numpy(w: int, h: int, dmin: int, dmax: int, seed: int, tiles: int = 10, bump: bool = False,
                   sigma_blur: float = 1.5):
    """The generator's definition in numpy (slow for large rigs)."""
    rnd = _Rand(seed)
    disp = disparity_map(rnd, h, w, dmin, dmax, tiles, bump)
    center = _texture(rnd, h, w, sigma_blur)
    fills = [_texture(rnd, h, w, sigma_blur) for _ in range(4)]
    right = _warp(center, disp, fills[0], 0, -1)
    top = _warp(center, disp, fills[1], 1, 0)
    left = _warp(center, disp, fills[2], 0, 1)
    bottom = _warp(center, disp, fills[3], -1, 0)
    views = [_sensor_noise(rnd, v) for v in (center, right, top, left, bottom)]
    return views, disp


# ---- the named workloads -------------------------------------------------------------------------

def rig_c1(seed: int = 1, native: bool = True):
    """640x480, maxdisp 192, 8-12 tiles with disparity 20-180."""
    rnd = _Rand(seed ^ 0x5151)
    return make_rig(640, 480, 20, 180, seed, tiles=rnd.int1(8, 12), native=native), 192


def rig_c2(seed: int = 2, native: bool = True):
    """1920x1080, maxdisp 256, 16 tiles + quadratic bump, disparity 10-240."""
    return make_rig(1920, 1080, 10, 240, seed, tiles=16, bump=True, native=native), 256


def rig_c5(seed: int = 5, native: bool = True):
    """Stress rig: 4096x3000, maxdisp 512, 32 tiles, disparity 20-500, sigma_blur 0.8."""
    return make_rig(4096, 3000, 20, 500, seed, tiles=32, sigma_blur=0.8, native=native), 512


def batch_shapes(n: int = 64, seed: int = 3):
    """Uneven batch: w ~ U[320,2448], h ~ U[240,2048] rounded to 16, dc in {64,128,192,256}, dc <= w/4."""
    rnd = _Rand(seed)
    shapes = []
    for _ in range(n):
        w = (rnd.int1(320, 2448) // 16) * 16
        h = (rnd.int1(240, 2048) // 16) * 16
        choices = [d for d in (64, 128, 192, 256) if d <= w // 4]
        dc = choices[rnd.int1(0, len(choices) - 1)]
        shapes.append((w, h, dc))
    return shapes


def rig_for_shape(w: int, h: int, dc: int, seed: int):
    dmax = max(min(dc - 16, int(dc * 0.94)), 8)
    dmin = max(dmax // 9, 2)
    return make_rig(w, h, dmin, dmax, seed, tiles=10), dc


SERVE_MIX = ((0.50, 640, 480, 128), (0.35, 1920, 1080, 256), (0.15, 2448, 2048, 256))
