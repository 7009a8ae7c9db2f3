// Masked multiview matching cost: the un-rotated, confidence-weighted sum of the four pair costs.
#include "sister_internal.h"

namespace sister {
namespace {

// multidsi of SisterMultiviewDisparities.hpp:255-277 at padded pixel (i, j):
//   M(d) = sum over used frames f of mask_f(i, j) * C_f(a_f, b_f, d)
// where (a_f, b_f) are the frame coordinates of (i, j) (hpp:259-261) and C_f is the pair's Hamming cell
// of census.cpp:54-146: 255 for frame rows 0..2, 0 for the two last rows (never written there), 255 for
// d > b, else popcount(Cc[a][b] ^ Cn[a][b-d]). Mode 0 uses all frames, 1 frames {0,2}, 2 frames {1,3}; mode 3 is the
// two-view doStereo volume (ad_census of hpp:135): frame 0 alone, without mask (masks may be null).
// The volume is stored with d-stride dp; entries d >= dc hold 0x7FFF, the aggregation's infinite cost
// (large enough never to win a minimum, small enough that packed 16-bit updates cannot wrap).
//
// A CTA computes a tile of 8 rows x TW columns of padded pixels (TW = 4 or 8). The transposed frames 1 and 3 read
// one frame row per tile column (a column of the padded image), so their neighbour census windows (dp + 10 words
// per tile column, 2 x TW windows) are staged in shared memory first and each word is fetched from L2/HBM once per
// tile instead of once per pixel; frames 0 and 2 read one contiguous stretch of their census row per tile row,
// which consecutive pixels share through L1. Each
// pixel's centre words and frame states (masked, constant row, or its column b) are staged too. Then warp w
// computes the TW pixels of tile row w, one at a time, lanes over d (lane l holds d = l + 32k, k < DPL). Frames whose
// column b >= dp-1 (most of them) need no per-lane d > b test; nearer the left edge the test is one warp-uniform
// branch per k. Summing the four frames' XOR words with carry-save adders before counting (5 popcounts instead
// of 8 per d) was slower in every form tried (2.2-3.5 ms against 1.40): the popcount pipe is not the limit.
constexpr int kCostWarps = 8; // warps per CTA; warp w computes tile rows w, w + 8, ...
constexpr int kNoCost = -3, kRow255 = -2, kRow0 = -1; // per-pixel frame states besides b >= 0
// words per staged frame row of a tile of RW rows (even): every b - d with d < dp for the tile's RW values of b, plus
// the rounding of the window's start down to an even column
__host__ __device__ inline int cost_win(int dp, int RW) { return dp + RW + 2; }
__host__ __device__ inline bool cost_in_mode(int mode, int f) {
    return mode == 0 || (mode == 1 && !(f & 1)) || (mode == 2 && (f & 1)) || (mode == 3 && f == 0);
}
// first (even) column of the window of tile row r of frame f: it covers every b - d with b in the tile and
// 0 <= d < dp
template <int TW, int RW>
__device__ __forceinline__ int cost_win0(const Geom &g, int f, int i0, int j0) {
    int c0;
    switch (f) {
    case 0: c0 = j0 - g.dp; break;                        // b = j
    case 2: c0 = g.Wp - j0 - (TW - 1) - g.dp; break;       // b = Wp-1-j
    case 1: c0 = g.Hp - i0 - (RW - 1) - g.dp; break;       // b = Hp-1-i
    default: c0 = i0 - g.dp; break;                         // b = i
    }
    return c0 & ~1;
}

template <int DPL, int TW, int RW>
__global__ void __launch_bounds__(256) masked_cost_kernel(const uint64_t *__restrict__ census,
                                                          const uint8_t *__restrict__ masks, Geom g, int mode,
                                                          uint16_t *__restrict__ cost) {
    extern __shared__ __align__(16) uint64_t win[]; // [frame 1, 3][tile column][cost_win(dp)]
    // per frame and tile pixel: the centre census word, or kNoCost when the pixel's frame is unused (out of the
    // mode or masked) and kRow255 / kRow0 when its frame row is constant
    __shared__ uint64_t ctr[4][RW * TW];
    __shared__ int fbs[4][RW * TW];
    const int nwin = cost_win(g.dp, RW);
    const int i0 = blockIdx.y * RW, j0 = blockIdx.x * TW;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int e = threadIdx.x; e < 4 * RW * TW; e += blockDim.x) {
        const int f = e / (RW * TW), t = e % (RW * TW);
        const int i = i0 + t / TW, j = j0 + t % TW;
        int fb = kNoCost;
        uint64_t c = 0;
        if (i < g.Hp && j < g.Wp && cost_in_mode(mode, f) &&
            (mode == 3 || masks[(size_t)f * g.plane + (size_t)i * g.Wp + j])) {
            int fa;
            switch (f) {
            case 0: fa = i; fb = j; break;
            case 2: fa = i; fb = g.Wp - 1 - j; break;
            case 1: fa = g.Wp - 1 - j; fb = g.Hp - 1 - i; break;
            default: fa = g.Wp - 1 - j; fb = i; break;
            }
            if (fa < 3) fb = kRow255; // whole frame row constant: 255 (rows 0..2) or 0 (never written)
            else if (fa >= g.frows(f) - 2) fb = kRow0;
            else c = census[(size_t)(2 * f) * g.plane + (size_t)fa * g.fcols(f) + fb];
        }
        fbs[f][t] = fb;
        ctr[f][t] = c;
    }
    // ---- stage the transposed frames' windows: warp w copies staged rows q = w, w+8, ... < 2 TW (frame 1 then 3,
    // tile column r = q % TW: frame row Wp-1-(j0+r)) with 16-byte asynchronous copies (windows start on even columns, frame rows on
    // 16-byte boundaries); columns outside the frame row are never read and stay unwritten. Frames 0 and 2 need one
    // contiguous stretch of their census row per tile row, read through L1 by the warps themselves.
    for (int q = w; q < 2 * TW; q += kCostWarps) {
        const int f = q < TW ? 1 : 3, r = q % TW;
        if (!cost_in_mode(mode, f)) continue;
        const int fa = g.Wp - 1 - (j0 + r);
        if (fa < 0 || fa >= g.frows(f)) continue;
        const int c0 = cost_win0<TW, RW>(g, f, i0, j0), fw = g.fcols(f);
        const uint64_t *src = census + (size_t)(2 * f + 1) * g.plane + (size_t)fa * fw;
        const uint32_t dst = (uint32_t)__cvta_generic_to_shared(win + (size_t)q * nwin);
        for (int u = lane; u < nwin / 2; u += 32) {
            const int col = c0 + 2 * u;
            if (col >= 0 && col < fw)
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * (uint32_t)u), "l"(src + col)
                             : "memory");
        }
    }
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    // ---- warp w: tile rows w, w + 8, ...
    const int D = g.dc;
    const int sw1 = -cost_win0<TW, RW>(g, 1, i0, j0), sw3 = TW * nwin - cost_win0<TW, RW>(g, 3, i0, j0);
    for (int rr = w; rr < RW; rr += kCostWarps) {
        const int i = i0 + rr;
        if (i >= g.Hp) return;
        // neighbour census row of each frame, indexed by the column b - d: frames 0 and 2 the global row i, frames 1 and
        // 3 the staged window of tile column jj
        const uint64_t *grow0 = census + (size_t)1 * g.plane + (size_t)i * g.Wp; // frame 0 (fa = i)
        const uint64_t *grow2 = census + (size_t)5 * g.plane + (size_t)i * g.Wp; // frame 2 (fa = i)
        for (int jj = 0; jj < TW; jj++) {
            const int j = j0 + jj;
            if (j >= g.Wp) break;
            const size_t p = (size_t)i * g.Wp + j;
            uint32_t acc[DPL];
#pragma unroll
            for (int k = 0; k < DPL; k++) acc[k] = 0;
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const int t = rr * TW + jj;
                const int fb = fbs[f][t]; // warp-uniform
                if (fb == kNoCost) continue;
                if (fb < 0) {
                    const uint32_t c = fb == kRow255 ? 255u : 0u;
#pragma unroll
                    for (int k = 0; k < DPL; k++) acc[k] += c;
                    continue;
                }
                const uint64_t cc = ctr[f][t];
                const uint64_t *wr = (f == 0) ? grow0 + fb
                                     : (f == 2) ? grow2 + fb
                                     : win + (jj * nwin + (f == 1 ? sw1 : sw3) + fb);
                if (fb >= g.dp - 1) { // every d of the stride has its word (d >= dc reads one that is never used)
#pragma unroll
                    for (int k = 0; k < DPL; k++) acc[k] += (uint32_t)__popcll(cc ^ wr[-(lane + 32 * k)]);
                } else {
                    // d = lane + 32k: every lane has d <= b below k = b / 32 and none above it (warp-uniform), so only
                    // that one k tests per lane; d > b costs 255 (census.cpp:74-78)
                    const int kb = fb >> 5;
#pragma unroll
                    for (int k = 0; k < DPL; k++) {
                        if (k < kb) {
                            acc[k] += (uint32_t)__popcll(cc ^ wr[-(lane + 32 * k)]);
                        } else if (k == kb) {
                            const int d = lane + 32 * k; // the load stays inside the row: column b - min(d, b) >= 0
                            const uint32_t h = (uint32_t)__popcll(cc ^ wr[-min(d, fb)]);
                            acc[k] += d <= fb ? h : 255u;
                        } else {
                            acc[k] += 255u;
                        }
                    }
                }
            }
            uint16_t *out = cost + p * g.dp;
            if (D == g.dp) { // every d of the stride is real
#pragma unroll
                for (int k = 0; k < DPL; k++) out[lane + 32 * k] = (uint16_t)acc[k];
            } else {
#pragma unroll
                for (int k = 0; k < DPL; k++) {
                    const int d = lane + 32 * k;
                    out[d] = d < D ? (uint16_t)acc[k] : (uint16_t)0x7FFF;
                }
            }
        }
    }
}

// tile width (columns) of the cost kernel for a d-stride: the staged windows take 2 x TW x (dp + 10) words. Four
// columns from dp = 256 up (17 KB at 256: eight CTAs per SM; 33 KB at 512: six), measured against eight: 1.10 ->
// 1.05 ms at 1920x1080/256, 14.2 -> 12.0 ms at 4096x3000/512; below 256 eight columns stay ahead by ~2%.
template <int DPL>
constexpr int cost_tw() { return 32 * DPL >= 256 ? 4 : 8; }
// tile rows (16 rows x 4 columns measured slower: 1.08 ms at 1920x1080/256, 13.1 ms at 4096x3000/512; 2 columns
// slower still)
template <int DPL>
constexpr int cost_rw() { return 8; }

template <int DPL>
void launch_cost_dpl(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                     cudaStream_t st) {
    constexpr int TW = cost_tw<DPL>(), RW = cost_rw<DPL>();
    dim3 grid((g.Wp + TW - 1) / TW, (g.Hp + RW - 1) / RW);
    const size_t smem = (size_t)2 * TW * cost_win(g.dp, RW) * sizeof(uint64_t);
    masked_cost_kernel<DPL, TW, RW><<<grid, 32 * kCostWarps, smem, st>>>(census, masks, g, mode, cost);
}

template <int DPL>
void set_cost_attr() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    constexpr int TW = cost_tw<DPL>(), RW = cost_rw<DPL>();
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, masked_cost_kernel<DPL, TW, RW>);
    cudaFuncSetAttribute(masked_cost_kernel<DPL, TW, RW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         optin - (int)fa.sharedSizeBytes); // the static part counts against the limit too
}

} // namespace

void launch_masked_cost(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                        cudaStream_t st) {
    switch (g.dpl) {
    case 2: launch_cost_dpl<2>(census, masks, g, mode, cost, st); break;
    case 4: launch_cost_dpl<4>(census, masks, g, mode, cost, st); break;
    case 6: launch_cost_dpl<6>(census, masks, g, mode, cost, st); break;
    case 8: launch_cost_dpl<8>(census, masks, g, mode, cost, st); break;
    case 12: launch_cost_dpl<12>(census, masks, g, mode, cost, st); break;
    default: launch_cost_dpl<16>(census, masks, g, mode, cost, st); break;
    }
}

void init_cost_kernels() {
    set_cost_attr<2>();
    set_cost_attr<4>();
    set_cost_attr<6>();
    set_cost_attr<8>();
    set_cost_attr<12>();
    set_cost_attr<16>();
    cudaGetLastError();
}

} // namespace sister
