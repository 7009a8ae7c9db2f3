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
// I(i+y, j+x) > I(i-y, j-x), y = -3..3 outer, x = -4..4 inner, shifted in from the right; bit 63 is the
// accumulator carry = bit 0 (last test, y=3, x=4) of the previous interior pixel in raster order,
// 0 for the first interior pixel (3,4). Non-interior pixels are 0.
// Block 32 x 8 pixels; shared tile covers rows [i0-3, i0+11) and columns [j0-5, j0+36).
__global__ void __launch_bounds__(256) census_kernel(const uint8_t *__restrict__ frames, Geom g,
                                                     uint64_t *__restrict__ census) {
    __shared__ uint8_t t[14][44];
    const int k = blockIdx.z, f = k >> 1;
    const int H = g.frows(f), W = g.fcols(f);
    const uint8_t *img = frames + (size_t)k * g.plane;
    uint64_t *out = census + (size_t)k * g.plane;
    const int i0 = blockIdx.y * 8, j0 = blockIdx.x * 32;
    if (i0 >= H || j0 >= W) return;
    const int tid = threadIdx.y * 32 + threadIdx.x;
    for (int e = tid; e < 14 * 41; e += 256) {
        const int r = e / 41, c = e % 41;
        const int y = i0 - 3 + r, x = j0 - 5 + c;
        t[r][c] = (y >= 0 && y < H && x >= 0 && x < W) ? img[(size_t)y * W + x] : 0;
    }
    __syncthreads();
    const int i = i0 + threadIdx.y, j = j0 + threadIdx.x;
    if (i >= H || j >= W) return;
    uint64_t v = 0;
    if (i >= 3 && i < H - 3 && j >= 4 && j < W - 4) {
        const int ty = threadIdx.y + 3, tx = threadIdx.x + 5;
#pragma unroll
        for (int y = -3; y <= 3; y++)
#pragma unroll
            for (int x = -4; x <= 4; x++) v = (v << 1) | (uint64_t)(t[ty + y][tx + x] > t[ty - y][tx - x]);
        uint64_t carry;
        if (j > 4) {
            carry = t[ty + 3][tx + 3] > t[ty - 3][tx - 5];
        } else if (i > 3) {
            // previous interior pixel is (i-1, W-5): its test reads (i+2, W-1) and (i-4, W-9)
            carry = img[(size_t)(i + 2) * W + (W - 1)] > img[(size_t)(i - 4) * W + (W - 9)];
        } else {
            carry = 0;
        }
        v |= carry << 63;
    }
    out[(size_t)i * W + j] = v;
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
    dim3 grid((mx + 31) / 32, (mx + 7) / 8, nimg);
    census_kernel<<<grid, dim3(32, 8), 0, st>>>(frames, g, census);
}

} // namespace sister
