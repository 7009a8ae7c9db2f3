// Masked multiview matching cost: the un-rotated, confidence-weighted sum of the four pair costs.
#include "sister_internal.h"

namespace sister {
namespace {

// multidsi of SisterMultiviewDisparities.hpp:255-277 at padded pixel (i, j):
//   M(d) = sum over used frames f of mask_f(i, j) * C_f(a_f, b_f, d)
// where (a_f, b_f) are the frame coordinates of (i, j) (hpp:259-261) and C_f is the pair's Hamming cell
// of census.cpp:54-146: 255 for frame rows 0..2, 0 for the two last rows (never written there), 255 for
// d > b, else popcount(Cc[a][b] ^ Cn[a][b-d]). Mode 0 uses all frames, 1 frames {0,2}, 2 frames {1,3}.
// The volume is stored with d-stride dp; entries d >= dc hold 0x7FFF, the aggregation's infinite cost
// (large enough never to win a minimum, small enough that packed 16-bit updates cannot wrap).
// One warp per pixel, lanes over d; 8 pixels of one row per CTA.
__global__ void __launch_bounds__(256) masked_cost_kernel(const uint64_t *__restrict__ census,
                                                          const uint8_t *__restrict__ masks, Geom g, int mode,
                                                          uint16_t *__restrict__ cost) {
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int i = blockIdx.y, j = blockIdx.x * 8 + wp;
    if (j >= g.Wp) return;
    const size_t p = (size_t)i * g.Wp + j;
    const int D = g.dc;

    bool use[4];
    int fa[4], fb[4], fh[4], fw[4];
    uint64_t cc[4];
    const uint64_t *cn[4];
#pragma unroll
    for (int f = 0; f < 4; f++) {
        const bool in_mode = (mode == 0) || (mode == 1 && !(f & 1)) || (mode == 2 && (f & 1));
        use[f] = in_mode && masks[(size_t)f * g.plane + p];
        switch (f) {
        case 0: fa[f] = i; fb[f] = j; break;
        case 2: fa[f] = i; fb[f] = g.Wp - 1 - j; break;
        case 1: fa[f] = g.Wp - 1 - j; fb[f] = g.Hp - 1 - i; break;
        default: fa[f] = g.Wp - 1 - j; fb[f] = i; break;
        }
        fh[f] = g.frows(f);
        fw[f] = g.fcols(f);
        const uint64_t *base = census + (size_t)(2 * f) * g.plane + (size_t)fa[f] * fw[f];
        cc[f] = use[f] ? base[fb[f]] : 0;
        cn[f] = census + (size_t)(2 * f + 1) * g.plane + (size_t)fa[f] * fw[f] + fb[f];
    }
    uint16_t *out = cost + p * g.dp;
    for (int d = lane; d < g.dp; d += 32) {
        uint32_t s = 0;
        if (d >= D) {
            s = 0x7FFFu;
        } else {
#pragma unroll
            for (int f = 0; f < 4; f++) {
                if (!use[f]) continue;
                uint32_t c;
                if (fa[f] < 3) c = 255;
                else if (fa[f] >= fh[f] - 2) c = 0;
                else if (d > fb[f]) c = 255;
                else c = (uint32_t)__popcll(cc[f] ^ __ldg(cn[f] - d));
                s += c;
            }
        }
        out[d] = (uint16_t)s;
    }
}

} // namespace

void launch_masked_cost(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                        cudaStream_t st) {
    dim3 grid((g.Wp + 7) / 8, g.Hp);
    masked_cost_kernel<<<grid, 256, 0, st>>>(census, masks, g, mode, cost);
}

} // namespace sister
