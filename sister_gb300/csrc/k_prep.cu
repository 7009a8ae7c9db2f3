// Preprocessing kernels: BGR->gray, replicate-padded rotated frame images, 9x7 census.
#include "sister_internal.h"

namespace sister {

int choose_dpl(int dc) {
    const int need = (dc + 31) / 32;
    for (int c : kDplChoices)
        if (c >= need) return c;
    return -1;
}

Geom make_geom(int w, int h, int dc) {
    Geom g;
    g.w = w;
    g.h = h;
    g.dc = dc;
    g.Wp = w + 2 * dc;
    g.Hp = h + 2 * dc;
    g.dpl = choose_dpl(dc);
    g.dp = 32 * g.dpl;
    g.plane = (size_t)g.Wp * g.Hp;
    return g;
}

namespace {

struct SrcPtrs {
    const uint8_t *p[5];
};

// cvtColor(BGR2GRAY) for 8-bit data (SisterMultiviewDisparities.hpp:29-33): OpenCV's published
// fixed-point weights 0.114/0.587/0.299 at 14 bits, rounded: (1868 B + 9617 G + 4899 R + 8192) >> 14.
// channels == 1 is a strided copy.
__global__ void to_gray_kernel(SrcPtrs src, int stride, int channels, int w, int h, uint8_t *__restrict__ dst) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    const int v = blockIdx.z;
    if (x >= w || y >= h) return;
    const uint8_t *row = src.p[v] + (size_t)y * stride;
    uint8_t g;
    if (channels == 3) {
        const uint32_t b = row[3 * x], gg = row[3 * x + 1], r = row[3 * x + 2];
        g = (uint8_t)((b * 1868u + gg * 9617u + r * 4899u + 8192u) >> 14);
    } else {
        g = row[x];
    }
    dst[(size_t)v * w * h + (size_t)y * w + x] = g;
}

// Frame images of doMultiStereo (SisterMultiviewDisparities.hpp:35-39, :54-70): replicate pad by dc, then
// frame 0 = identity, 1 = flip(transpose,-1), 2 = flip(.,1), 3 = flip(transpose,0). Image k = 2f is the
// center seen in frame f, k = 2f+1 its neighbour (right, top, left, bottom). 32x32 tiles staged through
// shared memory so that both the source rows and the (possibly transposed) destination rows are coalesced.
__global__ void frames_kernel(const uint8_t *__restrict__ views, Geom g, uint8_t *__restrict__ frames) {
    __shared__ uint8_t tile[32][33];
    const int k = blockIdx.z, f = k >> 1;
    const int src_view = (k & 1) ? (f + 1) : 0;
    const int rows = g.frows(f), cols = g.fcols(f);
    const uint8_t *src = views + (size_t)src_view * g.w * g.h;
    uint8_t *dst = frames + (size_t)k * g.plane;
    const int a0 = blockIdx.y * 32, b0 = blockIdx.x * 32;
    if (a0 >= rows || b0 >= cols) return;
    const int tx = threadIdx.x, ty = threadIdx.y; // 32 x 8
    if (f & 1) {
        // transposed frames: frame (a, b) reads padded (y, x) with x determined by a, y by b.
        // Load the source tile so that threads sweep padded x (= frame row index) contiguously.
        for (int s = ty; s < 32; s += 8) {
            const int b = b0 + s;    // frame column -> padded y
            const int a = a0 + tx;   // frame row    -> padded x (contiguous across tx)
            uint8_t v = 0;
            if (a < rows && b < cols) {
                const int y = (f == 1) ? (g.Hp - 1 - b) : b;
                const int x = g.Wp - 1 - a;
                const int yy = min(max(y - g.dc, 0), g.h - 1), xx = min(max(x - g.dc, 0), g.w - 1);
                v = src[(size_t)yy * g.w + xx];
            }
            tile[s][tx] = v; // tile[b - b0][a - a0]
        }
        __syncthreads();
        for (int s = ty; s < 32; s += 8) {
            const int a = a0 + s, b = b0 + tx;
            if (a < rows && b < cols) dst[(size_t)a * cols + b] = tile[tx][s];
        }
    } else {
        for (int s = ty; s < 32; s += 8) {
            const int a = a0 + s, b = b0 + tx;
            if (a < rows && b < cols) {
                const int x = (f == 2) ? (g.Wp - 1 - b) : b;
                const int yy = min(max(a - g.dc, 0), g.h - 1), xx = min(max(x - g.dc, 0), g.w - 1);
                dst[(size_t)a * cols + b] = src[(size_t)yy * g.w + xx];
            }
        }
    }
}

// censusTransform (census.cpp:38-51): for interior pixels i in [3,H-3), j in [4,W-4), 63 tests
// I(i+y, j+x) > I(i-y, j-x), y = -3..3 outer, x = -4..4 inner, shifted in from the right (test t ends at bit
// 62-t); bit 63 is the accumulator carry = bit 0 (last test, y=3, x=4) of the previous interior pixel in raster
// order, 0 for the first interior pixel (3,4). Non-interior pixels are 0.
// Each thread codes 4 consecutive pixels with byte-parallel (SWAR) compares of 32-bit words: for a test, the
// four pixels' operands are 4-byte windows of one tile row, cut from aligned words by funnel shifts, and
// a > b per byte is the high bit of maj(a, ~b, ~((b | 0x80..) - (a & 0x7f..))). Tests run from the last to the
// first, shifted into the top bit of each byte, so each group of 8 tests leaves one code byte per pixel, which a
// byte permute moves into place. Block 32 x 8 threads = 128 x 8 pixels; the shared tile holds rows
// [i0-3, i0+11) and columns [j0-8, j0+136) as words.
constexpr int kCW = 36; // tile words per row
__device__ __forceinline__ uint32_t win(const uint32_t *row, int c, int x) {
    // the 4 bytes at columns 4c + x .. 4c + x + 3 of a tile row (x in [-8, 7])
    const int q = c + (x >> 2), r = x & 3;
    return r ? __funnelshift_r(row[q], row[q + 1], 8 * r) : row[q];
}
__device__ __forceinline__ uint32_t gt4(uint32_t a, uint32_t b) {
    // high bit of each byte: a > b (unsigned), bytewise
    const uint32_t t = (b | 0x80808080u) - (a & 0x7F7F7F7Fu); // high bit: (b & 0x7f) >= (a & 0x7f)
    // ~maj(b, ~a, t) = maj(~b, a, ~t)
    const uint32_t nb = ~b, nt = ~t;
    return ((a & nb) | (a & nt) | (nb & nt)) & 0x80808080u;
}
__global__ void __launch_bounds__(256) census_kernel(const uint8_t *__restrict__ frames, Geom g,
                                                     uint64_t *__restrict__ census) {
    __shared__ uint32_t t[14][kCW];
    const int k = blockIdx.z, f = k >> 1;
    const int H = g.frows(f), W = g.fcols(f);
    const uint8_t *img = frames + (size_t)k * g.plane;
    uint64_t *out = census + (size_t)k * g.plane;
    const int i0 = blockIdx.y * 8, j0 = blockIdx.x * 128;
    if (i0 >= H || j0 >= W) return;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    // rows of a frame start on 4-byte boundaries (k * plane and W are multiples of 4) and W is a multiple of 4,
    // so each tile word is wholly inside or wholly outside the image
    for (int e = tid; e < 14 * kCW; e += 256) {
        const int r = e / kCW, c = e % kCW;
        const int y = i0 - 3 + r, x = j0 - 8 + 4 * c;
        t[r][c] = (y >= 0 && y < H && x >= 0 && x < W) ? *reinterpret_cast<const uint32_t *>(img + (size_t)y * W + x)
                                                       : 0u;
    }
    __syncthreads();
    const int i = i0 + threadIdx.y, j = j0 + 4 * threadIdx.x;
    if (i >= H || j >= W) return;
    uint32_t lo[4] = {0, 0, 0, 0}, hi[4] = {0, 0, 0, 0};
    if (i >= 3 && i < H - 3 && j + 3 >= 4 && j < W - 4) {
        const int ty = threadIdx.y + 3, c = 2 + threadIdx.x; // tile row of i, tile word of column j
        uint32_t acc = 0;
        int n = 0; // tests accumulated in acc
#pragma unroll
        for (int tt = 62; tt >= 0; tt--) {
            const int y = tt / 9 - 3, x = tt % 9 - 4;
            const uint32_t gt = gt4(win(t[ty + y], c, x), win(t[ty - y], c, -x));
            acc = ((acc >> 1) & 0x7F7F7F7Fu) | gt;
            n++;
            if (n == 8) {
                // tests tt+7 .. tt: code bits 8G .. 8G+7 with G = (62 - (tt + 7)) / 8
                const int G = (62 - (tt + 7)) / 8;
#pragma unroll
                for (int p = 0; p < 4; p++) {
                    // byte p of acc into byte G % 4 of lo (G < 4) or hi
                    const int sel = (0x3210 & ~(0xF << (4 * (G & 3)))) | ((4 + p) << (4 * (G & 3)));
                    if (G < 4) lo[p] = __byte_perm(lo[p], acc, sel);
                    else hi[p] = __byte_perm(hi[p], acc, sel);
                }
                acc = 0;
                n = 0;
            }
        }
        // the last 7 tests (6 .. 0) sit in bits 1..7 of each byte: code bits 56..62 = byte 3 of hi, bits 0..6
        acc >>= 1;
#pragma unroll
        for (int p = 0; p < 4; p++) hi[p] = __byte_perm(hi[p], acc & 0x7F7F7F7Fu, (0x0210) | ((4 + p) << 12));
        // carries: the last test (y=3, x=4) of pixels j-1 .. j+2: I(i+3, j+3+p) > I(i-3, j-5+p)
        const uint32_t cy = gt4(win(t[ty + 3], c, 3), win(t[ty - 3], c, -5));
#pragma unroll
        for (int p = 0; p < 4; p++) hi[p] |= (cy >> (8 * p + 7)) << 31;
        if (j == 4) {
            // previous interior pixel of (i, 4) is (i-1, W-5): its test reads (i+2, W-1) and (i-4, W-9)
            const uint32_t cp = (i > 3) ? (img[(size_t)(i + 2) * W + (W - 1)] > img[(size_t)(i - 4) * W + (W - 9)]) : 0u;
            hi[0] = (hi[0] & 0x7FFFFFFFu) | (cp << 31);
        }
        // pixels outside [4, W-4) are 0
#pragma unroll
        for (int p = 0; p < 4; p++)
            if (j + p < 4 || j + p >= W - 4) lo[p] = hi[p] = 0;
    }
    uint4 *o = reinterpret_cast<uint4 *>(out + (size_t)i * W + j);
    o[0] = make_uint4(lo[0], hi[0], lo[1], hi[1]);
    o[1] = make_uint4(lo[2], hi[2], lo[3], hi[3]);
}

} // namespace

void launch_to_gray(const uint8_t *const src[5], int stride, int channels, int w, int h, uint8_t *views_dev,
                    cudaStream_t st) {
    SrcPtrs s;
    for (int v = 0; v < 5; v++) s.p[v] = src[v];
    dim3 grid((w + 127) / 128, h, 5);
    to_gray_kernel<<<grid, 128, 0, st>>>(s, stride, channels, w, h, views_dev);
}

void launch_frames(const uint8_t *views_dev, const Geom &g, uint8_t *frames, cudaStream_t st) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    dim3 grid((mx + 31) / 32, (mx + 31) / 32, 8);
    frames_kernel<<<grid, dim3(32, 8), 0, st>>>(views_dev, g, frames);
}

void launch_census(const uint8_t *frames, const Geom &g, uint64_t *census, cudaStream_t st, int nimg) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    dim3 grid((mx + 127) / 128, (mx + 7) / 8, nimg);
    census_kernel<<<grid, dim3(32, 8), 0, st>>>(frames, g, census);
}

} // namespace sister
