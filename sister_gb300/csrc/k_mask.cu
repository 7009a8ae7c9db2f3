// Confidence-mask kernels: per-pair WTA-left/right from census words, the reference's in-place
// (row-recursive) 3x3 median, LR check and the per-pair masks in padded original coordinates.
#include "sister_internal.h"

namespace sister {
namespace {

// WTALeft_SSE / WTARight_SSE with uniqueness 1 (postprocess.cpp:74-315) on a pair's Hamming volume
// (census.cpp:54-146), without materialising the volume. Both reduce to the lowest-index argmin:
//   L(j) = argmin_{d <= min(j, D-1)} popc(Cc[j] ^ Cn[j-d])
//   R(j) = argmin_{k <= min(D-1, W-1-j)} popc(Cc[j+k] ^ Cn[j])
// Rows 0..2 (all 255) and rows H-2, H-1 (never written, defined 0) have constant costs: argmin 0.
// One CTA per frame row; both census rows staged in shared memory. Keys pack (cost << 16 | d) so a
// plain unsigned min yields the lowest-index minimum.
__global__ void __launch_bounds__(256) pair_wta_kernel(const uint64_t *__restrict__ census, Geom g,
                                                       uint16_t *__restrict__ wta) {
    extern __shared__ uint64_t srow[];
    const int f = blockIdx.y;
    const int H = g.frows(f), W = g.fcols(f), D = g.dc;
    const int i = blockIdx.x;
    if (i >= H) return;
    uint16_t *L = wta + (size_t)(2 * f) * g.plane + (size_t)i * W;
    uint16_t *R = wta + (size_t)(2 * f + 1) * g.plane + (size_t)i * W;
    if (i < 3 || i >= H - 2) {
        for (int j = threadIdx.x; j < W; j += blockDim.x) {
            L[j] = 0;
            R[j] = 0;
        }
        return;
    }
    uint64_t *cc = srow, *cn = srow + W;
    const uint64_t *gc = census + (size_t)(2 * f) * g.plane + (size_t)i * W;
    const uint64_t *gn = census + (size_t)(2 * f + 1) * g.plane + (size_t)i * W;
    for (int j = threadIdx.x; j < W; j += blockDim.x) {
        cc[j] = gc[j];
        cn[j] = gn[j];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < W; j += blockDim.x) {
        const uint64_t a = cc[j];
        const int endl = min(j, D - 1);
        uint32_t best = 0xFFFFFFFFu;
        for (int d = 0; d <= endl; d++) best = min(best, ((uint32_t)__popcll(a ^ cn[j - d]) << 16) | (uint32_t)d);
        L[j] = (uint16_t)(best & 0xFFFFu);
        const uint64_t b = cn[j];
        const int endr = min(D - 1, W - 1 - j);
        best = 0xFFFFFFFFu;
        for (int k = 0; k <= endr; k++) best = min(best, ((uint32_t)__popcll(cc[j + k] ^ b) << 16) | (uint32_t)k);
        R[j] = (uint16_t)(best & 0xFFFFu);
    }
}

// shared ring length for the median sweep: a power of two >= 2W
__host__ __device__ inline int median_ring(int W) {
    int r = 1;
    while (r < 2 * W) r <<= 1;
    return r;
}

__device__ __forceinline__ void cswap(uint32_t &a, uint32_t &b) {
    const uint32_t t = min(a, b);
    b = max(a, b);
    a = t;
}

// Median of nine by the 19-exchange selection network; exact on integers.
__device__ __forceinline__ uint32_t med9(uint32_t v0, uint32_t v1, uint32_t v2, uint32_t v3, uint32_t v4, uint32_t v5,
                                         uint32_t v6, uint32_t v7, uint32_t v8) {
    cswap(v1, v2); cswap(v4, v5); cswap(v7, v8);
    cswap(v0, v1); cswap(v3, v4); cswap(v6, v7);
    cswap(v1, v2); cswap(v4, v5); cswap(v7, v8);
    cswap(v0, v3); cswap(v5, v8); cswap(v4, v7);
    cswap(v3, v6); cswap(v1, v4); cswap(v2, v5);
    cswap(v4, v7); cswap(v4, v2); cswap(v6, v4);
    cswap(v4, v2);
    return v4;
}

// median3x3_SSE(a, a, W, H) in place (postprocess.cpp:15-71 as called at SisterMultiviewDisparities.hpp:198
// and siblings). Over the flattened array of N = W*H: out[x] = in[x] for x < W and x >= N-W-4;
// out[W] = 0; for W < x < N-W-4, out[x] = med9(out[x-W-1], out[x-W], out[x-W+1], in[x-1], in[x], in[x+1],
// in[x+W-1], in[x+W], in[x+W+1]) where the first three were already filtered in the same sweep.
// out[x] depends only on positions <= x-W+1, so chunks of W-1 consecutive positions are independent:
// one CTA sweeps the chunks in order, keeping the last 2W outputs in a shared ring.
__global__ void __launch_bounds__(1024) median_kernel(const uint16_t *__restrict__ wta, Geom g,
                                                      uint16_t *__restrict__ med) {
    extern __shared__ uint16_t ring[]; // ring[x & mask] = out[x] for the last 2W positions
    const int k = blockIdx.x, f = k >> 1;
    const int H = g.frows(f), W = g.fcols(f);
    const int N = W * H;
    const uint16_t *in = wta + (size_t)k * g.plane;
    uint16_t *out = med + (size_t)k * g.plane;
    const int mask = median_ring(W) - 1;
    // head: x < W unchanged, x == W -> 0
    for (int x = threadIdx.x; x <= W; x += blockDim.x) {
        const uint16_t v = (x < W) ? in[x] : (uint16_t)0;
        out[x] = v;
        ring[x & mask] = v;
    }
    // tail: x >= N-W-4 unchanged
    for (int x = N - W - 4 + threadIdx.x; x < N; x += blockDim.x) out[x] = in[x];
    __syncthreads();
    const int end = N - W - 4;
    for (int s = W + 1; s < end; s += W - 1) {
        const int e = min(s + W - 1, end);
        for (int x = s + threadIdx.x; x < e; x += blockDim.x) {
            const uint32_t v = med9(ring[(x - W - 1) & mask], ring[(x - W) & mask], ring[(x - W + 1) & mask],
                                    __ldg(in + x - 1), __ldg(in + x), __ldg(in + x + 1),
                                    __ldg(in + x + W - 1), __ldg(in + x + W), __ldg(in + x + W + 1));
            ring[x & mask] = (uint16_t)v;
            out[x] = (uint16_t)v;
        }
        __syncthreads();
    }
}

// doLRCheck(L, R, W, H, 5) (postprocess.cpp:318-341) and the mask loops of SisterMultiviewDisparities.hpp:201-251:
// keep = L <= j && |L - R[j-L]| <= 5; mask = keep && L > 0 && j >= dc; written in padded original
// coordinates (frame 2: (i, Wp-1-j); frame 1: transpose + flip(-1); frame 3: transpose + flip(1)).
__global__ void lrc_mask_kernel(const uint16_t *__restrict__ med, Geom g, uint8_t *__restrict__ masks) {
    const int f = blockIdx.z;
    const int H = g.frows(f), W = g.fcols(f);
    const int b = blockIdx.x * blockDim.x + threadIdx.x, a = blockIdx.y;
    if (a >= H || b >= W) return;
    const uint16_t *L = med + (size_t)(2 * f) * g.plane + (size_t)a * W;
    const uint16_t *R = med + (size_t)(2 * f + 1) * g.plane + (size_t)a * W;
    const int base = L[b];
    bool keep = false;
    if (base <= b) {
        const int diff = base - (int)R[b - base];
        keep = diff <= 5 && diff >= -5;
    }
    const uint8_t m = (keep && base > 0 && b >= g.dc) ? 1 : 0;
    int i, j;
    switch (f) {
    case 0: i = a; j = b; break;
    case 2: i = a; j = g.Wp - 1 - b; break;
    case 1: i = g.Hp - 1 - b; j = g.Wp - 1 - a; break;
    default: i = b; j = g.Wp - 1 - a; break;
    }
    masks[(size_t)f * g.plane + (size_t)i * g.Wp + j] = m;
}

} // namespace

void init_mask_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncSetAttribute(pair_wta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(median_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaGetLastError();
}

void launch_pair_wta(const uint64_t *census, const Geom &g, uint16_t *wta, cudaStream_t st) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    const size_t smem = 2 * (size_t)mx * sizeof(uint64_t);
    pair_wta_kernel<<<dim3(mx, 4), 256, smem, st>>>(census, g, wta);
}

void launch_median(const uint16_t *wta, const Geom &g, uint16_t *med, cudaStream_t st) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    const size_t smem = (size_t)median_ring(mx) * sizeof(uint16_t);
    median_kernel<<<8, 1024, smem, st>>>(wta, g, med);
}

void launch_lrc_mask(const uint16_t *med, const Geom &g, uint8_t *masks, cudaStream_t st) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    lrc_mask_kernel<<<dim3((mx + 255) / 256, mx, 4), 256, 0, st>>>(med, g, masks);
}

} // namespace sister
