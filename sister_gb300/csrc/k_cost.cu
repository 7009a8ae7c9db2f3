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
// One warp per pixel, lanes over d (lane l holds d = l + 32k, k < DPL); 8 pixels of one row per CTA, CTAs ordered
// row-fastest. The
// frame loop is outside the d loop so that the DPL census loads of one frame are independent and issue
// back to back (the transposed frames' words come from L2).
template <int DPL>
__global__ void __launch_bounds__(256) masked_cost_kernel(const uint64_t *__restrict__ census,
                                                          const uint8_t *__restrict__ masks, Geom g, int mode,
                                                          uint16_t *__restrict__ cost) {
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    const int i = blockIdx.x, j = blockIdx.y * 8 + wp;
    if (j >= g.Wp) return;
    const size_t p = (size_t)i * g.Wp + j;
    const int D = g.dc;
    uint32_t acc[DPL];
#pragma unroll
    for (int k = 0; k < DPL; k++) acc[k] = 0;
#pragma unroll
    for (int f = 0; f < 4; f++) {
        const bool in_mode = (mode == 0) || (mode == 1 && !(f & 1)) || (mode == 2 && (f & 1)) || (mode == 3 && f == 0);
        if (!in_mode || (mode != 3 && !masks[(size_t)f * g.plane + p])) continue; // warp-uniform
        int fa, fb;
        switch (f) {
        case 0: fa = i; fb = j; break;
        case 2: fa = i; fb = g.Wp - 1 - j; break;
        case 1: fa = g.Wp - 1 - j; fb = g.Hp - 1 - i; break;
        default: fa = g.Wp - 1 - j; fb = i; break;
        }
        const int fh = g.frows(f), fw = g.fcols(f);
        if (fa < 3 || fa >= fh - 2) { // whole frame row constant: 255 (rows 0..2) or 0 (never written)
            const uint32_t c = fa < 3 ? 255u : 0u;
#pragma unroll
            for (int k = 0; k < DPL; k++) acc[k] += c;
            continue;
        }
        const uint64_t cc = census[(size_t)(2 * f) * g.plane + (size_t)fa * fw + fb];
        const uint64_t *cn = census + (size_t)(2 * f + 1) * g.plane + (size_t)fa * fw + fb;
        uint64_t wv[DPL];
#pragma unroll
        for (int k = 0; k < DPL; k++) {
            const int d = lane + 32 * k;
            wv[k] = (d <= fb && d < D) ? __ldg(cn - d) : 0;
        }
#pragma unroll
        for (int k = 0; k < DPL; k++) {
            const int d = lane + 32 * k;
            acc[k] += d > fb ? 255u : (uint32_t)__popcll(cc ^ wv[k]);
        }
    }
    uint16_t *out = cost + p * g.dp;
#pragma unroll
    for (int k = 0; k < DPL; k++) {
        const int d = lane + 32 * k;
        out[d] = d < D ? (uint16_t)acc[k] : (uint16_t)0x7FFF;
    }
}

} // namespace

void launch_masked_cost(const uint64_t *census, const uint8_t *masks, const Geom &g, int mode, uint16_t *cost,
                        cudaStream_t st) {
    // rows fastest: consecutive CTAs share the transposed frames' census rows (a frame-1/3 row is a padded
    // column), which then come from L1/L2 instead of being gathered again
    dim3 grid(g.Hp, (g.Wp + 7) / 8);
    switch (g.dpl) {
    case 2: masked_cost_kernel<2><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    case 4: masked_cost_kernel<4><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    case 6: masked_cost_kernel<6><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    case 8: masked_cost_kernel<8><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    case 12: masked_cost_kernel<12><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    default: masked_cost_kernel<16><<<grid, 256, 0, st>>>(census, masks, g, mode, cost); break;
    }
}

} // namespace sister
