// 8-path semi-global aggregation (sgm.cpp:26-455, called as sgm(.., 7, 17, 8) at
// SisterMultiviewDisparities.hpp:280) fused with the final winner-take-all (hpp:283), crop and *255 (hpp:111-118).
//
// The reference runs two raster passes; each pass updates four paths per pixel:
//   r0 from (i, j-dj), r1 from (i-di, j-dj), r2 from (i-di, j), r3 from (i-di, j+dj)
// with P1 = 7 and a constant P2 = 100 (adaptP2 with alpha = 0, sgm.cpp:15-22, :34-35).
// In pass coordinates (row r, column q; pass 1 mirrors both axes) the dependencies are
// (r, q-1), (r-1, q-1), (r-1, q), (r-1, q+1), so pixel (r, q) can run at wavefront step 2r + q.
//
// Work decomposition: a band of R consecutive rows per CTA, one warp per row, 32 lanes x DPL
// disparities per pixel. At step t warp w handles column q = t - 2w, so the row above is always two
// columns ahead; its r1/r2/r3 states travel through a 4-slot shared-memory ring. The last row of a band
// hands its states to the next band through global memory with a published progress counter (the only
// inter-CTA wait; it is bounded and reports kErrTimeout instead of hanging). CTAs are persistent and
// take bands in increasing order, so every wait points to a lower band.
//
// Pass 0 stores the pass sum (u16) for every pixel; pass 1 adds its own paths and reduces over d.
#include "sister_internal.h"

#include <algorithm>

namespace sister {
namespace {

constexpr uint32_t INF = 0xFFFFu;
constexpr unsigned FULL = 0xFFFFFFFFu;

template <bool CG>
__device__ __forceinline__ uint4 ld4(const uint16_t *p) {
    if constexpr (CG) return __ldcg(reinterpret_cast<const uint4 *>(p));
    else return *reinterpret_cast<const uint4 *>(p);
}
template <bool CG>
__device__ __forceinline__ uint2 ld2(const uint16_t *p) {
    if constexpr (CG) return __ldcg(reinterpret_cast<const uint2 *>(p));
    else return *reinterpret_cast<const uint2 *>(p);
}
template <bool CG>
__device__ __forceinline__ uint32_t ld1(const uint16_t *p) {
    if constexpr (CG) return __ldcg(reinterpret_cast<const unsigned int *>(p));
    else return *reinterpret_cast<const uint32_t *>(p);
}

// N consecutive u16 starting at p (aligned to the vector width used) -> N u32
template <int N, bool CG = false>
__device__ __forceinline__ void ld16(const uint16_t *p, uint32_t (&o)[N]) {
    if constexpr (N % 8 == 0) {
#pragma unroll
        for (int k = 0; k < N / 8; k++) {
            const uint4 v = ld4<CG>(p + 8 * k);
            o[8 * k + 0] = v.x & 0xFFFFu; o[8 * k + 1] = v.x >> 16;
            o[8 * k + 2] = v.y & 0xFFFFu; o[8 * k + 3] = v.y >> 16;
            o[8 * k + 4] = v.z & 0xFFFFu; o[8 * k + 5] = v.z >> 16;
            o[8 * k + 6] = v.w & 0xFFFFu; o[8 * k + 7] = v.w >> 16;
        }
    } else if constexpr (N % 4 == 0) {
#pragma unroll
        for (int k = 0; k < N / 4; k++) {
            const uint2 v = ld2<CG>(p + 4 * k);
            o[4 * k + 0] = v.x & 0xFFFFu; o[4 * k + 1] = v.x >> 16;
            o[4 * k + 2] = v.y & 0xFFFFu; o[4 * k + 3] = v.y >> 16;
        }
    } else if constexpr (N % 2 == 0) {
#pragma unroll
        for (int k = 0; k < N / 2; k++) {
            const uint32_t v = ld1<CG>(p + 2 * k);
            o[2 * k] = v & 0xFFFFu;
            o[2 * k + 1] = v >> 16;
        }
    } else {
#pragma unroll
        for (int k = 0; k < N; k++) o[k] = CG ? (uint32_t)__ldcg(p + k) : (uint32_t)p[k];
    }
}

__device__ __forceinline__ uint32_t pk(uint32_t lo, uint32_t hi) { return min(lo, INF) | (min(hi, INF) << 16); }

// N values clamped to 0xFFFF, stored as consecutive u16
template <int N>
__device__ __forceinline__ void st16(uint16_t *p, const uint32_t (&v)[N]) {
    if constexpr (N % 8 == 0) {
#pragma unroll
        for (int k = 0; k < N / 8; k++)
            reinterpret_cast<uint4 *>(p)[k] = make_uint4(pk(v[8 * k], v[8 * k + 1]), pk(v[8 * k + 2], v[8 * k + 3]),
                                                         pk(v[8 * k + 4], v[8 * k + 5]), pk(v[8 * k + 6], v[8 * k + 7]));
    } else if constexpr (N % 4 == 0) {
#pragma unroll
        for (int k = 0; k < N / 4; k++)
            reinterpret_cast<uint2 *>(p)[k] = make_uint2(pk(v[4 * k], v[4 * k + 1]), pk(v[4 * k + 2], v[4 * k + 3]));
    } else if constexpr (N % 2 == 0) {
#pragma unroll
        for (int k = 0; k < N / 2; k++) reinterpret_cast<uint32_t *>(p)[k] = pk(v[2 * k], v[2 * k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < N; k++) p[k] = (uint16_t)min(v[k], INF);
    }
}

// One path update of the remaining lines (sgm.cpp:278-383), per disparity d of this lane:
//   L(d) = C(d) + min(Lp(d), Lp(d-1)+P1, Lp(d+1)+P1, minLp+P2) - minLp
// Lp(-1) = Lp(D) = 0xFFFF. The reference uses u16 saturating arithmetic; for real disparities no
// intermediate reaches 0xFFFF (L <= C + 100 <= 1120), values derived from 0xFFFF never win the min
// against minLp + 100, so plain u32 arithmetic is identical. Entries of padded disparities grow to at
// most 0xFFFF + 100 and are clamped whenever they are stored.
template <int DPL>
__device__ __forceinline__ uint32_t path_step(const uint32_t (&Lp)[DPL], uint32_t minLp, const uint32_t (&c)[DPL],
                                              uint32_t (&Ln)[DPL], int lane) {
    uint32_t left = __shfl_up_sync(FULL, Lp[DPL - 1], 1);
    uint32_t right = __shfl_down_sync(FULL, Lp[0], 1);
    if (lane == 0) left = INF;
    if (lane == 31) right = INF;
    const uint32_t p2 = minLp + 100u;
    uint32_t mn = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < DPL; k++) {
        const uint32_t lo = k ? Lp[k - 1] : left;
        const uint32_t hi = (k + 1 < DPL) ? Lp[k + 1] : right;
        const uint32_t m = min(min(lo, hi) + 7u, min(Lp[k], p2));
        const uint32_t v = c[k] + m - minLp;
        Ln[k] = v;
        mn = min(mn, v);
    }
    return mn;
}

__device__ __forceinline__ uint32_t warp_min2(uint32_t v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = __vminu2(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ uint32_t warp_min(uint32_t v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <int DPL, int PASS>
__global__ void __launch_bounds__(DPL >= 12 ? 256 : 512) sgm_kernel(const SgmArgs a) {
    extern __shared__ __align__(16) uint16_t smem[];
    const int R = a.R, W = a.W, H = a.H, dp = a.dp, D = a.D;
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int d0 = lane * DPL;
    const int slot = 3 * dp; // r1 | r2 | r3 of one pixel
    uint16_t *ring = smem;                         // [R][4][3*dp]
    uint16_t *rmin = smem + (size_t)R * 4 * slot;  // [R][4][4]

    for (int band = blockIdx.x; band < a.nbands; band += gridDim.x) {
        const int r = band * R + wi;
        const bool rowok = r < H;
        const int i = PASS ? (H - 1 - r) : r;
        const bool publish = (wi == R - 1) && (band + 1 < a.nbands);
        uint32_t r0[DPL];
        uint32_t r0min = 0;
        unsigned seen = 0;
#pragma unroll
        for (int k = 0; k < DPL; k++) r0[k] = INF;
        const int T = W + 2 * (R - 1);
        for (int t = 0; t < T; t++) {
            const int q = t - 2 * wi;
            if (rowok && q >= 0 && q < W) {
                const int j = PASS ? (W - 1 - q) : q;
                const size_t pix = (size_t)i * W + j;
                uint32_t c[DPL];
                ld16<DPL>(a.cost + pix * dp + d0, c);
                uint32_t n1[DPL], n2[DPL], n3[DPL], g[DPL];
                uint32_t mn0, mn1, mn2, mn3;
                if (r == 0) {
                    // First line of the pass (sgm.cpp:103-207): C' = (C == 255 ? 0 : C); r1..r3 take C'
                    // with min C'; r0 starts as C' and then runs the recurrence in int32 truncated to
                    // 8 bits (saturate_cast<uint16>(uint8), types.h:28); the sum gets r0 alone.
                    uint32_t cp[DPL];
                    uint32_t mc = 0xFFFFFFFFu;
#pragma unroll
                    for (int k = 0; k < DPL; k++) {
                        cp[k] = (c[k] == 255u) ? 0u : c[k]; // padded entries (0xFFFF) stay infinite
                        mc = min(mc, cp[k]);
                    }
                    if (q == 0) {
#pragma unroll
                        for (int k = 0; k < DPL; k++) g[k] = cp[k];
                        mn0 = mc;
                    } else {
                        uint32_t left = __shfl_up_sync(FULL, r0[DPL - 1], 1);
                        uint32_t right = __shfl_down_sync(FULL, r0[0], 1);
                        if (lane == 0) left = INF;
                        if (lane == 31) right = INF;
                        const uint32_t p2 = r0min + 100u;
                        mn0 = 0xFFFFFFFFu;
#pragma unroll
                        for (int k = 0; k < DPL; k++) {
                            const uint32_t lo = k ? r0[k - 1] : left;
                            const uint32_t hi = (k + 1 < DPL) ? r0[k + 1] : right;
                            const uint32_t m = min(min(lo, hi) + 7u, min(r0[k], p2));
                            const uint32_t v = (d0 + k < D) ? ((cp[k] + m - r0min) & 0xFFu) : INF;
                            g[k] = v;
                            mn0 = min(mn0, v);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < DPL; k++) {
                        r0[k] = g[k];
                        n1[k] = n2[k] = n3[k] = cp[k];
                    }
                    mn1 = mn2 = mn3 = mc;
                } else {
                    // states of the row above: r1 at q-1, r2 at q, r3 at q+1 (missing columns: 0xFFFF, min 0)
                    const uint16_t *s1 = nullptr, *s2, *s3 = nullptr;
                    uint32_t m1 = 0, m2, m3 = 0;
                    uint32_t p1[DPL], pp2[DPL], p3[DPL];
                    if (wi > 0) {
                        const uint16_t *base = ring + (size_t)(wi - 1) * 4 * slot;
                        const uint16_t *mb = rmin + (wi - 1) * 16;
                        if (q > 0) { s1 = base + ((q - 1) & 3) * slot; m1 = mb[((q - 1) & 3) * 4 + 0]; }
                        s2 = base + (q & 3) * slot + dp;
                        m2 = mb[(q & 3) * 4 + 1];
                        if (q + 1 < W) { s3 = base + ((q + 1) & 3) * slot + 2 * dp; m3 = mb[((q + 1) & 3) * 4 + 2]; }
                        if (s1) ld16<DPL>(s1 + d0, p1);
                        ld16<DPL>(s2 + d0, pp2);
                        if (s3) ld16<DPL>(s3 + d0, p3);
                    } else {
                        // first row of a band > 0: wait until the previous band published column q+1
                        const unsigned need = (unsigned)min(q + 2, W);
                        if (seen < need) {
                            unsigned n = 0;
                            for (;;) {
                                const unsigned v = ld_acquire(a.progress + band - 1);
                                if (v >= need) { seen = v; break; }
                                if (ld_acquire(a.err) != kErrNone || ++n > a.spin_limit) {
                                    atomicCAS(a.err, kErrNone, kErrTimeout);
                                    seen = 0xFFFFFFFFu;
                                    break;
                                }
                                __nanosleep(200);
                            }
                        }
                        const uint16_t *gb = a.bnd + (size_t)(band - 1) * W * slot;
                        const uint16_t *gm = a.bmin + (size_t)(band - 1) * W * 4;
                        if (q > 0) { s1 = gb + (size_t)(q - 1) * slot; m1 = __ldcg(gm + (size_t)(q - 1) * 4 + 0); }
                        s2 = gb + (size_t)q * slot + dp;
                        m2 = __ldcg(gm + (size_t)q * 4 + 1);
                        if (q + 1 < W) { s3 = gb + (size_t)(q + 1) * slot + 2 * dp; m3 = __ldcg(gm + (size_t)(q + 1) * 4 + 2); }
                        if (s1) ld16<DPL, true>(s1 + d0, p1);
                        ld16<DPL, true>(s2 + d0, pp2);
                        if (s3) ld16<DPL, true>(s3 + d0, p3);
                    }
                    if (!s1) {
#pragma unroll
                        for (int k = 0; k < DPL; k++) p1[k] = INF;
                    }
                    if (!s3) {
#pragma unroll
                        for (int k = 0; k < DPL; k++) p3[k] = INF;
                    }
                    if (q == 0) {
                        // r0 restarts every row from Lp = 0, minLp = 0 (sgm.cpp:215-216)
#pragma unroll
                        for (int k = 0; k < DPL; k++) r0[k] = (d0 + k < D) ? 0u : INF;
                        r0min = 0;
                    }
                    uint32_t n0[DPL];
                    mn0 = path_step<DPL>(r0, r0min, c, n0, lane);
                    mn1 = path_step<DPL>(p1, m1, c, n1, lane);
                    mn2 = path_step<DPL>(pp2, m2, c, n2, lane);
                    mn3 = path_step<DPL>(p3, m3, c, n3, lane);
#pragma unroll
                    for (int k = 0; k < DPL; k++) {
                        r0[k] = n0[k];
                        g[k] = n0[k] + n1[k] + n2[k] + n3[k];
                    }
                }
                const uint32_t a01 = warp_min2(min(mn0, INF) | (min(mn1, INF) << 16));
                const uint32_t a23 = warp_min2(min(mn2, INF) | (min(mn3, INF) << 16));
                r0min = a01 & 0xFFFFu;
                // hand r1/r2/r3 of (r, q) to the row below
                if (wi + 1 < R) {
                    uint16_t *dst = ring + ((size_t)wi * 4 + (q & 3)) * slot;
                    st16<DPL>(dst + d0, n1);
                    st16<DPL>(dst + dp + d0, n2);
                    st16<DPL>(dst + 2 * dp + d0, n3);
                    if (lane == 0) {
                        uint16_t *mb = rmin + wi * 16 + (q & 3) * 4;
                        mb[0] = (uint16_t)(a01 >> 16);
                        mb[1] = (uint16_t)(a23 & 0xFFFFu);
                        mb[2] = (uint16_t)(a23 >> 16);
                    }
                } else if (publish) {
                    uint16_t *dst = a.bnd + ((size_t)band * W + q) * slot;
                    st16<DPL>(dst + d0, n1);
                    st16<DPL>(dst + dp + d0, n2);
                    st16<DPL>(dst + 2 * dp + d0, n3);
                    if (lane == 0) {
                        uint16_t *mb = a.bmin + ((size_t)band * W + q) * 4;
                        mb[0] = (uint16_t)(a01 >> 16);
                        mb[1] = (uint16_t)(a23 & 0xFFFFu);
                        mb[2] = (uint16_t)(a23 >> 16);
                    }
                    if ((q & 3) == 3 || q == W - 1) {
                        __threadfence();
                        __syncwarp();
                        if (lane == 0) st_release(a.progress + band, (unsigned)(q + 1));
                    }
                }
                if (PASS == 0) {
                    st16<DPL>(a.sum0 + pix * dp + d0, g);
                } else {
                    // pass 1 adds to the pass-0 sum (first line: plain u16 add, sgm.cpp:132,:187; else
                    // saturating, :390 -- neither wraps nor saturates for real disparities), then the
                    // final WTALeft: lowest d <= min(j, dc-1) of the total (hpp:283, postprocess.cpp:74-185).
                    uint32_t s0[DPL];
                    ld16<DPL>(a.sum0 + pix * dp + d0, s0);
                    uint32_t best = 0xFFFFFFFFu;
#pragma unroll
                    for (int k = 0; k < DPL; k++) {
                        const int d = d0 + k;
                        const uint32_t s = (s0[k] + g[k]) & 0xFFFFu;
                        if (d < D && d <= j) best = min(best, (s << 16) | (uint32_t)d);
                    }
                    best = warp_min(best);
                    if (lane == 0) {
                        const uint32_t disp = best & 0xFFFFu;
                        if (a.disp) a.disp[pix] = (uint16_t)disp;
                        if (a.out) {
                            const int oi = i - a.dc, oj = j - a.dc;
                            if (oi >= 0 && oi < a.h && oj >= 0 && oj < a.w)
                                a.out[(size_t)oi * a.w + oj] = (uint16_t)min(disp * 255u, INF);
                        }
                    }
                }
            }
            __syncthreads();
        }
    }
}

template <int DPL>
void set_attrs(int optin) {
    cudaFuncSetAttribute(sgm_kernel<DPL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(sgm_kernel<DPL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <int DPL>
cudaError_t run(const Geom &g, SgmArgs a, cudaStream_t st, int device) {
    const int threads = a.R * 32;
    const size_t smem = (size_t)a.R * 4 * 3 * g.dp * sizeof(uint16_t) + (size_t)a.R * 16 * sizeof(uint16_t);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    for (int pass = 0; pass < 2; pass++) {
        const void *fn = pass ? (const void *)sgm_kernel<DPL, 1> : (const void *)sgm_kernel<DPL, 0>;
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) return cudaErrorInvalidConfiguration;
        const int grid = std::min(a.nbands, per_sm * sms);
        e = cudaMemsetAsync(a.progress, 0, (size_t)a.nbands * sizeof(unsigned), st);
        if (e != cudaSuccess) return e;
        void *args[] = {(void *)&a};
        e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, smem, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

} // namespace

void init_sgm_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    set_attrs<1>(optin); set_attrs<2>(optin); set_attrs<3>(optin); set_attrs<4>(optin);
    set_attrs<6>(optin); set_attrs<8>(optin); set_attrs<12>(optin); set_attrs<16>(optin);
    cudaGetLastError();
}

int sgm_rows_per_band(const Geom &g, int num_sms) {
    const int maxR = g.dpl >= 12 ? 8 : 16;
    int R = (g.Hp + num_sms - 1) / num_sms;
    return std::max(2, std::min(R, maxR));
}

size_t sgm_bnd_elems(const Geom &g, int num_sms) {
    const int R = sgm_rows_per_band(g, num_sms);
    const size_t nb = (size_t)(g.Hp + R - 1) / R;
    return nb * g.Wp * 3 * (size_t)g.dp;
}

cudaError_t launch_sgm(const Geom &g, SgmArgs a, cudaStream_t st, int device) {
    switch (g.dpl) {
    case 1: return run<1>(g, a, st, device);
    case 2: return run<2>(g, a, st, device);
    case 3: return run<3>(g, a, st, device);
    case 4: return run<4>(g, a, st, device);
    case 6: return run<6>(g, a, st, device);
    case 8: return run<8>(g, a, st, device);
    case 12: return run<12>(g, a, st, device);
    case 16: return run<16>(g, a, st, device);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace sister
