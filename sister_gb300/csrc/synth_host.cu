// Host-side synthetic rig generator: the same integer algorithm as sister_gb300/synth.py (make_rig), byte
// for byte, in C for speed (benchmark batches hold 64 rigs of up to 2448x2048). Test infrastructure for
// workloads only; no GPU code. See synth.py for the description of the scene model.
#include "sister_gb300.h"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {

struct Rand {
    uint64_t seed;
    uint64_t stream = 0;
    explicit Rand(long long s) : seed((uint64_t)s & 0xFFFFFFFFull) {}
    // n integers uniform in [lo, hi] from the splitmix64 counter hash of (seed, stream, index), index = 1..n
    // (synth.py _splitmix / _Rand.ints)
    void ints(long long lo, long long hi, size_t n, std::vector<int64_t> &out) {
        stream++;
        const uint64_t base = seed * 0x9E3779B97F4A7C15ull + stream * 0xD1B54A32D192ED03ull;
        const uint64_t span = (uint64_t)(hi - lo + 1);
        out.resize(n);
        auto mix = [&](size_t i) {
            uint64_t z = base + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            return z ^ (z >> 31);
        };
        if ((span & (span - 1)) == 0) { // power of two: the remainder is a mask
            for (size_t i = 0; i < n; i++) out[i] = (int64_t)(mix(i) & (span - 1)) + lo;
        } else {
            for (size_t i = 0; i < n; i++) out[i] = (int64_t)(mix(i) % span) + lo;
        }
    }
    long long int1(long long lo, long long hi) {
        std::vector<int64_t> v;
        ints(lo, hi, 1, v);
        return v[0];
    }
};

// floor division / arithmetic shift as numpy int64 does
inline int64_t fdiv(int64_t a, int64_t b) {
    int64_t q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}
inline int64_t ashr16(int64_t v) { return fdiv(v, 65536); }

const int kK15[] = {16, 117, 554, 1684, 3280, 4096, 3280, 1684, 554, 117, 16};
const int kK08[] = {4, 180, 1875, 4096, 1875, 180, 4};

void blur(const std::vector<int64_t> &a, int h, int w, const int *k, int nk, std::vector<int64_t> &out) {
    const int r = nk / 2;
    int64_t s = 0;
    for (int t = 0; t < nk; t++) s += k[t];
    std::vector<int64_t> hb((size_t)h * w);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int64_t acc = 0;
            for (int t = 0; t < nk; t++) {
                int xx = x + t - r;
                xx = xx < 0 ? 0 : (xx >= w ? w - 1 : xx);
                acc += (int64_t)k[t] * a[(size_t)y * w + xx];
            }
            hb[(size_t)y * w + x] = fdiv(acc + s / 2, s);
        }
    out.resize((size_t)h * w);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int64_t acc = 0;
            for (int t = 0; t < nk; t++) {
                int yy = y + t - r;
                yy = yy < 0 ? 0 : (yy >= h ? h - 1 : yy);
                acc += (int64_t)k[t] * hb[(size_t)yy * w + x];
            }
            out[(size_t)y * w + x] = fdiv(acc + s / 2, s);
        }
}

void texture(Rand &rnd, int h, int w, bool s15, std::vector<int64_t> &out) {
    std::vector<int64_t> noise;
    rnd.ints(0, 255, (size_t)h * w, noise);
    std::vector<int64_t> b;
    blur(noise, h, w, s15 ? kK15 : kK08, s15 ? 11 : 7, b);
    int64_t lo = b[0], hi = b[0];
    for (int64_t v : b) {
        lo = v < lo ? v : lo;
        hi = v > hi ? v : hi;
    }
    const int64_t den = (hi - lo) > 1 ? (hi - lo) : 1;
    out.resize(b.size());
    for (size_t i = 0; i < b.size(); i++) out[i] = fdiv((b[i] - lo) * 255, den);
}

struct Plane {
    int64_t d0, gx, gy, cx, cy;
    int64_t at(int y, int x) const { return d0 * 65536 + gx * (x - cx) + gy * (y - cy); }
};
Plane plane(Rand &rnd, int h, int w, int dmin, int dmax) {
    Plane p;
    p.d0 = rnd.int1(dmin, dmax);
    p.gx = rnd.int1(-3276, 3276);
    p.gy = rnd.int1(-3276, 3276);
    p.cx = rnd.int1(0, w - 1);
    p.cy = rnd.int1(0, h - 1);
    return p;
}

void disparity_map(Rand &rnd, int h, int w, int dmin, int dmax, int tiles, bool bump, std::vector<int64_t> &d) {
    std::vector<int64_t> fx((size_t)h * w);
    const Plane bg = plane(rnd, h, w, dmin, (dmin + dmax) / 2);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) fx[(size_t)y * w + x] = bg.at(y, x);
    auto imax = [](long long a, long long b) { return a > b ? a : b; };
    for (int t = 0; t < tiles; t++) {
        const long long tw = rnd.int1(imax(w / 12, 4), imax(w / 3, 5));
        const long long th = rnd.int1(imax(h / 12, 4), imax(h / 3, 5));
        const long long x0 = rnd.int1(0, imax(w - tw, 0));
        const long long y0 = rnd.int1(0, imax(h - th, 0));
        const Plane p = plane(rnd, h, w, dmin, dmax);
        for (long long y = y0; y < y0 + th && y < h; y++)
            for (long long x = x0; x < x0 + tw && x < w; x++) {
                int64_t &v = fx[(size_t)y * w + x];
                const int64_t pv = p.at((int)y, (int)x);
                v = pv > v ? pv : v;
            }
    }
    if (bump) {
        const long long cx = rnd.int1(w / 4, 3 * w / 4), cy = rnd.int1(h / 4, 3 * h / 4);
        const long long mn = h < w ? h : w;
        const long long rad = rnd.int1(mn / 6, mn / 3);
        const long long amp = rnd.int1(5, 30);
        for (int y = 0; y < h; y++)
            for (int x = 0; x < w; x++) {
                const int64_t r2 = (int64_t)(x - cx) * (x - cx) + (int64_t)(y - cy) * (y - cy);
                if (r2 < rad * rad) fx[(size_t)y * w + x] += fdiv(amp * 65536 * (rad * rad - r2), rad * rad);
            }
    }
    d.resize(fx.size());
    for (size_t i = 0; i < fx.size(); i++) {
        int64_t v = ashr16(fx[i] + 32768);
        d[i] = v < dmin ? dmin : (v > dmax ? dmax : v);
    }
}

// forward warp out(y + dy*d, x + dx*d) = center(y, x); larger d wins, equal d: the later source in raster
// order wins (numpy's repeated-index assignment order); holes <- fill
void warp(const std::vector<int64_t> &center, const std::vector<int64_t> &disp, const std::vector<int64_t> &fill, int h,
          int w, int dy, int dx, std::vector<int64_t> &out) {
    std::vector<int64_t> best((size_t)h * w, -1);
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const int64_t d = disp[(size_t)y * w + x];
            const int64_t ty = y + dy * d, tx = x + dx * d;
            if (ty < 0 || ty >= h || tx < 0 || tx >= w) continue;
            int64_t &b = best[(size_t)ty * w + tx];
            b = d > b ? d : b;
        }
    out = fill;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const int64_t d = disp[(size_t)y * w + x];
            const int64_t ty = y + dy * d, tx = x + dx * d;
            if (ty < 0 || ty >= h || tx < 0 || tx >= w) continue;
            const size_t t = (size_t)ty * w + tx;
            if (best[t] == d) out[t] = center[(size_t)y * w + x];
        }
}

void sensor_noise(Rand &rnd, const std::vector<int64_t> &img, uint8_t *dst) {
    const size_t n = img.size();
    std::vector<int64_t> acc(n, 0), v;
    for (int k = 0; k < 12; k++) {
        rnd.ints(0, 65535, n, v);
        for (size_t i = 0; i < n; i++) acc[i] += v[i];
    }
    for (size_t i = 0; i < n; i++) {
        const int64_t noise = (acc[i] - 12 * 32768) * 2;
        int64_t q = ashr16(img[i] * 65536 + noise + 32768);
        dst[i] = (uint8_t)(q < 0 ? 0 : (q > 255 ? 255 : q));
    }
}

} // namespace

extern "C" SISTER_API int sister_synth_rig(int w, int h, int dmin, int dmax, long long seed, int tiles, int bump,
                                           int sigma_tenths, uint8_t *views, int32_t *disparity) {
    if (w < 1 || h < 1 || dmin > dmax || tiles < 0 || !views || (sigma_tenths != 15 && sigma_tenths != 8))
        return SISTER_EINVAL;
    Rand rnd(seed);
    std::vector<int64_t> disp, center, fills[4];
    disparity_map(rnd, h, w, dmin, dmax, tiles, bump != 0, disp);
    texture(rnd, h, w, sigma_tenths == 15, center);
    for (auto &f : fills) texture(rnd, h, w, sigma_tenths == 15, f);
    std::vector<int64_t> vw[5];
    vw[0] = center;
    warp(center, disp, fills[0], h, w, 0, -1, vw[1]); // right
    warp(center, disp, fills[1], h, w, 1, 0, vw[2]);  // top
    warp(center, disp, fills[2], h, w, 0, 1, vw[3]);  // left
    warp(center, disp, fills[3], h, w, -1, 0, vw[4]); // bottom
    const size_t n = (size_t)w * h;
    for (int v = 0; v < 5; v++) sensor_noise(rnd, vw[v], views + v * n);
    if (disparity)
        for (size_t i = 0; i < n; i++) disparity[i] = (int32_t)disp[i];
    return SISTER_OK;
}
