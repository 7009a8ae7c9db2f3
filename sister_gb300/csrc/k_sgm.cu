// 8-path semi-global aggregation (sgm.cpp:26-455, called as sgm(.., 7, 17, 8) at
// SisterMultiviewDisparities.hpp:280) fused with the final winner-take-all (hpp:283), crop and *255 (hpp:111-118).
//
// The reference runs two raster passes; each pass updates four paths per pixel:
//   r0 from (i, j-dj), r1 from (i-di, j-dj), r2 from (i-di, j), r3 from (i-di, j+dj)
// with P1 = 7 and a constant P2 = 100 (adaptP2 with alpha = 0, sgm.cpp:15-22, :34-35). In pass
// coordinates (row r, column q; pass 1 mirrors both axes) pixel (r, q) depends on (r, q-1), (r-1, q-1),
// (r-1, q) and (r-1, q+1): a wavefront in which every row trails the row above by two columns.
//
// Work decomposition
//   * one warp per image row ("compute warp"), 32 lanes x DPL disparities, sweeping q = 0..W-1;
//   * R consecutive rows form a band = one CTA; CS consecutive bands form a group = one thread-block
//     cluster; clusters are persistent and take groups in increasing order;
//   * a row hands the r1/r2/r3 states of each pixel to the row below through a 4-slot ring of state
//     records guarded by full/empty mbarriers. Inside a CTA the ring is local shared memory; between
//     CTAs of a cluster the producer writes straight into the consumer CTA's shared memory (DSMEM) and
//     arrives on its barrier remotely; between clusters a publisher warp copies the last row of the group
//     to global memory and releases a progress counter, and a fetcher warp of the next group polls it and
//     fills that group's first ring. Compute warps never fence or poll global memory.
//   * the cost volume (and, in pass 1, the pass-0 sum) are prefetched per warp with cp.async, three
//     pixels ahead.
// Arithmetic is packed u16x2 (__vminu2 / __vadd2 / __vsub2, all full-rate on sm_103). Real values stay
// below 1221 so nothing wraps; "infinite" entries (missing columns, disparities >= dc) are 0x7FFF and stay
// below 0x8064 after any update, so they never win a minimum and never overflow 16 bits.
// Every wait is bounded: on expiry the device error flag is raised and the kernel finishes.
#include "sister_internal.h"

#include <algorithm>

namespace sister {

constexpr int kCR = 8;    // cost (and pass-0 sum) prefetch ring slots per compute warp
constexpr int kPF = 3;    // prefetch distance in pixels
constexpr int kK = 4;     // slots of a row-to-row state ring (power of two)

// One state record: r1 | r2 | r3 (dp u16 each) | minima m1 m2 m3 (+5 pad) -> 6dp + 16 bytes.
__host__ __device__ inline int rec_u16(int dp) { return 3 * dp + 8; }

struct SgmSmem {
    size_t bars, cring, sring, rings, total;
};
// rings 0..R: ring c feeds compute warp c (c < R) or the publisher (c == R)
__host__ __device__ inline SgmSmem sgm_smem(int R, int dp, int pass) {
    SgmSmem L{};
    size_t o = 0;
    L.bars = o;
    o += ((size_t)(R + 1) * kK * 2 + kK) * 8; // full/empty per ring slot, then E_out[kK]
    o = (o + 15) & ~(size_t)15;
    L.cring = o;
    o += (size_t)R * kCR * dp * 2;
    L.sring = o;
    if (pass) o += (size_t)R * kCR * dp * 2;
    L.rings = o;
    o += (size_t)(R + 1) * kK * rec_u16(dp) * 2;
    L.total = o;
    return L;
}

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t INF2 = 0x7FFF7FFFu;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t sptr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t cta_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_idx() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t mapa(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void cp16(void *sdst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sptr(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint32_t a) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive_local(uint32_t a) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
// Bounded wait for phase parity `par`. CLUSTER selects cluster-scope acquire, needed only when the
// arriving threads live in another CTA of the cluster; CTA scope is much cheaper.
template <bool CLUSTER>
__device__ __forceinline__ void mbar_wait(uint32_t a, uint32_t par, const SgmArgs &g) {
    for (unsigned n = 0;; n++) {
        uint32_t ok;
        if constexpr (CLUSTER)
            asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2; "
                         "selp.u32 %0, 1, 0, p; }"
                         : "=r"(ok)
                         : "r"(a), "r"(par)
                         : "memory");
        else
            asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2; "
                         "selp.u32 %0, 1, 0, p; }"
                         : "=r"(ok)
                         : "r"(a), "r"(par)
                         : "memory");
        if (ok) return;
        if ((n & 1023u) == 1023u && (ld_acquire(g.err) != kErrNone || n > g.spin_limit)) {
            atomicCAS(g.err, kErrNone, kErrTimeout);
            return;
        }
    }
}

// NP consecutive 32-bit words (2*NP u16) from shared memory / to shared memory (local or DSMEM)
template <int NP>
__device__ __forceinline__ void lds(const uint16_t *p, uint32_t (&o)[NP]) {
    if constexpr (NP % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 4; k++) {
            const uint4 v = reinterpret_cast<const uint4 *>(p)[k];
            o[4 * k] = v.x; o[4 * k + 1] = v.y; o[4 * k + 2] = v.z; o[4 * k + 3] = v.w;
        }
    } else if constexpr (NP % 2 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 2; k++) {
            const uint2 v = reinterpret_cast<const uint2 *>(p)[k];
            o[2 * k] = v.x; o[2 * k + 1] = v.y;
        }
    } else {
#pragma unroll
        for (int k = 0; k < NP; k++) o[k] = reinterpret_cast<const uint32_t *>(p)[k];
    }
}
template <int NP>
__device__ __forceinline__ void sts_local(uint16_t *p, const uint32_t (&v)[NP]) {
    if constexpr (NP % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 4; k++)
            reinterpret_cast<uint4 *>(p)[k] = make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
    } else if constexpr (NP % 2 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 2; k++) reinterpret_cast<uint2 *>(p)[k] = make_uint2(v[2 * k], v[2 * k + 1]);
    } else {
#pragma unroll
        for (int k = 0; k < NP; k++) reinterpret_cast<uint32_t *>(p)[k] = v[k];
    }
}
template <int NP>
__device__ __forceinline__ void sts_cluster(uint32_t a, const uint32_t (&v)[NP]) {
    if constexpr (NP % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 4; k++)
            asm volatile("st.shared::cluster.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a + 16 * k), "r"(v[4 * k]),
                         "r"(v[4 * k + 1]), "r"(v[4 * k + 2]), "r"(v[4 * k + 3])
                         : "memory");
    } else if constexpr (NP % 2 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 2; k++)
            asm volatile("st.shared::cluster.v2.u32 [%0], {%1, %2};" ::"r"(a + 8 * k), "r"(v[2 * k]), "r"(v[2 * k + 1])
                         : "memory");
    } else {
#pragma unroll
        for (int k = 0; k < NP; k++) asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(a + 4 * k), "r"(v[k]) : "memory");
    }
}

// ---------------------------------------------------------------- packed path update
__device__ __forceinline__ uint32_t perm_hi_lo(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
__device__ __forceinline__ uint32_t hmin(uint32_t v) { return min(v & 0xFFFFu, v >> 16); }

// remaining-lines update of one path (sgm.cpp:278-383) for this lane's DPL = 2*NP disparities:
//   L(d) = C(d) + min(Lp(d), Lp(d-1)+7, Lp(d+1)+7, minLp+100) - minLp; returns the lane's minimum
template <int NP>
__device__ __forceinline__ uint32_t path_step(const uint32_t (&P)[NP], uint32_t minLp, const uint32_t (&C)[NP],
                                              uint32_t (&Ln)[NP], int lane) {
    uint32_t left = __shfl_up_sync(FULL, P[NP - 1], 1);
    uint32_t right = __shfl_down_sync(FULL, P[0], 1);
    if (lane == 0) left = INF2;
    if (lane == 31) right = INF2;
    const uint32_t m2 = minLp * 0x00010001u;
    const uint32_t p2 = (minLp + 100u) * 0x00010001u;
    uint32_t xprev = perm_hi_lo(left, P[0]); // (Lp[d-1], Lp[d]) of the first pair
    uint32_t mn = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        const uint32_t x = perm_hi_lo(P[k], (k + 1 < NP) ? P[k + 1] : right); // (Lp[d+1], Lp[d+2])
        const uint32_t t = __vadd2(__vminu2(xprev, x), 0x00070007u);
        const uint32_t m = __vminu2(t, __vminu2(P[k], p2));
        const uint32_t v = __vadd2(C[k], __vsub2(m, m2));
        Ln[k] = v;
        mn = __vminu2(mn, v);
        xprev = x;
    }
    return hmin(mn);
}

// ---------------------------------------------------------------- the kernel
template <int DPL, int PASS>
__global__ void __launch_bounds__(DPL >= 12 ? 320 : 576) sgm_kernel(const SgmArgs a) {
    constexpr int NP = DPL / 2;
    extern __shared__ __align__(16) unsigned char smem[];
    const int R = a.R, W = a.W, H = a.H, dp = a.dp, D = a.D, CS = a.cs;
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int d0 = lane * DPL;
    const int rec = rec_u16(dp);
    const uint32_t rank = cta_rank();
    const SgmSmem L = sgm_smem(R, dp, PASS);
    const uint32_t bars = sptr(smem + L.bars);
    auto full_bar = [&](int c, int s) { return bars + (uint32_t)((c * kK + s) * 2) * 8u; };
    auto empty_bar = [&](int c, int s) { return bars + (uint32_t)((c * kK + s) * 2 + 1) * 8u; };
    auto eout_bar = [&](int s) { return bars + (uint32_t)((R + 1) * kK * 2 + s) * 8u; };
    uint16_t *rings = reinterpret_cast<uint16_t *>(smem + L.rings);
    auto ring_slot = [&](int c, int s) { return rings + (size_t)(c * kK + s) * rec; };
    const int nbar = (R + 1) * kK * 2 + kK;

    // halves holding disparities >= dc are infinite
    uint32_t padm[NP];
#pragma unroll
    for (int k = 0; k < NP; k++)
        padm[k] = ((d0 + 2 * k < D) ? 0u : 0x0000FFFFu) | ((d0 + 2 * k + 1 < D) ? 0u : 0xFFFF0000u);

    bool first_group = true;
    for (int grp = (int)cluster_idx(); grp < a.ngroups; grp += (int)cluster_count()) {
        const int band = grp * CS + (int)rank;
        if (threadIdx.x == 0) {
            for (int k = 0; k < nbar; k++) {
                const uint32_t b = bars + 8u * k;
                if (!first_group) mbar_inval(b);
                mbar_init(b, 32);
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        first_group = false;
        cluster_sync();
        if (band < a.nbands) {
            const bool has_fetcher = (rank == 0) && (band > 0);
            const bool has_publisher = (rank == (uint32_t)(CS - 1)) && (band + 1 < a.nbands);
            if (wi < R) {
                // ======================================================= compute warp: row r
                const int r = band * R + wi;
                if (r < H) {
                    const int i = PASS ? (H - 1 - r) : r;
                    const bool first_line = (r == 0);
                    const size_t rowbase = (size_t)i * W;
                    // input: ring wi of this CTA; for warp 0 of a non-leading CTA it is written by CTA rank-1
                    const bool remote_in = (wi == 0) && !first_line && !has_fetcher;
                    // output: 0 none, 1 local ring wi+1 (next warp or the publisher), 2 ring 0 of CTA rank+1
                    int omode = 0;
                    if (r + 1 < H) omode = (wi + 1 < R || has_publisher) ? 1 : 2;
                    uint16_t *cring = reinterpret_cast<uint16_t *>(smem + L.cring) + (size_t)wi * kCR * dp;
                    uint16_t *sring = reinterpret_cast<uint16_t *>(smem + L.sring) + (size_t)wi * kCR * dp;
                    const int chunks = dp / 8;
                    auto issue = [&](int x) {
                        if (x < W) {
                            const size_t pix = rowbase + (PASS ? (W - 1 - x) : x);
                            const uint16_t *src = a.cost + pix * dp;
                            uint16_t *dst = cring + (size_t)(x & (kCR - 1)) * dp;
                            for (int c = lane; c < chunks; c += 32) cp16(dst + 8 * c, src + 8 * c);
                            if (PASS) {
                                const uint16_t *s2 = a.sum0 + pix * dp;
                                uint16_t *d2 = sring + (size_t)(x & (kCR - 1)) * dp;
                                for (int c = lane; c < chunks; c += 32) cp16(d2 + 8 * c, s2 + 8 * c);
                            }
                        }
                        cp_commit();
                    };
                    for (int x = 0; x < kPF; x++) issue(x);

                    uint32_t r0[NP];
                    uint32_t r0min = 0;
#pragma unroll
                    for (int k = 0; k < NP; k++) r0[k] = INF2;

                    for (int q = 0; q < W; q++) {
                        cp_wait<kPF - 1>();
                        __syncwarp();
                        if (!first_line) {
                            const uint32_t par1 = ((q + 1) / kK) & 1;
                            if (remote_in) {
                                if (q == 0) mbar_wait<true>(full_bar(wi, 0), 0, a);
                                if (q + 1 < W) mbar_wait<true>(full_bar(wi, (q + 1) & (kK - 1)), par1, a);
                            } else {
                                if (q == 0) mbar_wait<false>(full_bar(wi, 0), 0, a);
                                if (q + 1 < W) mbar_wait<false>(full_bar(wi, (q + 1) & (kK - 1)), par1, a);
                            }
                        }
                        issue(q + kPF);
                        const int j = PASS ? (W - 1 - q) : q;
                        uint32_t c[NP];
                        lds<NP>(cring + (size_t)(q & (kCR - 1)) * dp + d0, c);
                        uint32_t n1[NP], n2[NP], n3[NP], gsum[NP];
                        uint32_t mn0, mn1, mn2, mn3;
                        if (first_line) {
                            // First line of the pass (sgm.cpp:103-207): C' = (C == 255 ? 0 : C); r1..r3 take
                            // C' with min C'; r0 starts as C' and then runs the recurrence in int32 truncated to
                            // 8 bits (saturate_cast<uint16>(uint8), types.h:28); the sum gets r0 alone.
                            uint32_t cp[NP];
                            uint32_t mc = 0xFFFFFFFFu;
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                cp[k] = c[k] & ~__vcmpeq2(c[k], 0x00FF00FFu);
                                mc = __vminu2(mc, cp[k]);
                            }
                            mc = hmin(mc);
                            if (q == 0) {
#pragma unroll
                                for (int k = 0; k < NP; k++) gsum[k] = cp[k];
                                mn0 = mc;
                            } else {
                                uint32_t tmp[NP];
                                path_step<NP>(r0, r0min, cp, tmp, lane);
                                uint32_t mnv = 0xFFFFFFFFu;
#pragma unroll
                                for (int k = 0; k < NP; k++) {
                                    const uint32_t v = (tmp[k] & 0x00FF00FFu & ~padm[k]) | (INF2 & padm[k]);
                                    gsum[k] = v;
                                    mnv = __vminu2(mnv, v);
                                }
                                mn0 = hmin(mnv);
                            }
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                r0[k] = gsum[k];
                                n1[k] = n2[k] = n3[k] = cp[k];
                            }
                            mn1 = mn2 = mn3 = mc;
                        } else {
                            // states of the row above: r1 at q-1, r2 at q, r3 at q+1 (missing column: inf, min 0)
                            uint32_t p1[NP], p2v[NP], p3[NP];
                            uint32_t m1 = 0, m3 = 0;
                            if (q > 0) {
                                const uint16_t *s = ring_slot(wi, (q - 1) & (kK - 1));
                                lds<NP>(s + d0, p1);
                                m1 = s[3 * dp + 0];
                            } else {
#pragma unroll
                                for (int k = 0; k < NP; k++) p1[k] = INF2;
                            }
                            const uint16_t *s2 = ring_slot(wi, q & (kK - 1));
                            lds<NP>(s2 + dp + d0, p2v);
                            const uint32_t m2 = s2[3 * dp + 1];
                            if (q + 1 < W) {
                                const uint16_t *s3 = ring_slot(wi, (q + 1) & (kK - 1));
                                lds<NP>(s3 + 2 * dp + d0, p3);
                                m3 = s3[3 * dp + 2];
                            } else {
#pragma unroll
                                for (int k = 0; k < NP; k++) p3[k] = INF2;
                            }
                            if (q == 0) { // r0 restarts every row from Lp = 0, minLp = 0 (sgm.cpp:215-216)
#pragma unroll
                                for (int k = 0; k < NP; k++) r0[k] = INF2 & padm[k];
                                r0min = 0;
                            }
                            uint32_t n0[NP];
                            mn0 = path_step<NP>(r0, r0min, c, n0, lane);
                            mn1 = path_step<NP>(p1, m1, c, n1, lane);
                            mn2 = path_step<NP>(p2v, m2, c, n2, lane);
                            mn3 = path_step<NP>(p3, m3, c, n3, lane);
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                r0[k] = n0[k];
                                gsum[k] = __vadd2(__vadd2(n0[k], n1[k]), __vadd2(n2[k], n3[k]));
                            }
                            // the slot of column q-1 is no longer needed by this row
                            if (q >= 1) {
                                const int s = (q - 1) & (kK - 1);
                                if (remote_in) mbar_arrive_remote(mapa(eout_bar(s), rank - 1));
                                else mbar_arrive_local(empty_bar(wi, s));
                            }
                        }
                        r0min = __reduce_min_sync(FULL, mn0);
                        // hand r1/r2/r3 of (r, q) to the row below
                        if (omode) {
                            const uint32_t v1 = __reduce_min_sync(FULL, mn1);
                            const uint32_t v2 = __reduce_min_sync(FULL, mn2);
                            const uint32_t v3 = __reduce_min_sync(FULL, mn3);
                            const int s = q & (kK - 1);
                            if (omode == 1) {
                                if (q >= kK) mbar_wait<false>(empty_bar(wi + 1, s), ((q / kK) - 1) & 1, a);
                                uint16_t *dst = ring_slot(wi + 1, s);
                                sts_local<NP>(dst + d0, n1);
                                sts_local<NP>(dst + dp + d0, n2);
                                sts_local<NP>(dst + 2 * dp + d0, n3);
                                if (lane == 0)
                                    *reinterpret_cast<uint2 *>(dst + 3 * dp) = make_uint2(v1 | (v2 << 16), v3);
                                mbar_arrive_local(full_bar(wi + 1, s));
                            } else {
                                if (q >= kK) mbar_wait<true>(eout_bar(s), ((q / kK) - 1) & 1, a);
                                const uint32_t dst = mapa(sptr(ring_slot(0, s)), rank + 1);
                                sts_cluster<NP>(dst + 2u * d0, n1);
                                sts_cluster<NP>(dst + 2u * (dp + d0), n2);
                                sts_cluster<NP>(dst + 2u * (2 * dp + d0), n3);
                                if (lane == 0)
                                    asm volatile("st.shared::cluster.v2.u32 [%0], {%1, %2};" ::"r"(dst + 6u * dp),
                                                 "r"(v1 | (v2 << 16)), "r"(v3)
                                                 : "memory");
                                mbar_arrive_remote(mapa(full_bar(0, s), rank + 1));
                            }
                        }
                        const size_t pix = rowbase + j;
                        if (PASS == 0) {
                            sts_local<NP>(a.sum0 + pix * dp + d0, gsum); // generic store to global
                        } else {
                            // pass 1 adds to the pass-0 sum (first line: plain u16 add, sgm.cpp:132,:187; else
                            // saturating, :390 -- neither wraps nor saturates for real disparities), then the
                            // final WTALeft: lowest d <= min(j, dc-1) of the total (hpp:283, postprocess.cpp:74-185).
                            uint32_t s0[NP];
                            lds<NP>(sring + (size_t)(q & (kCR - 1)) * dp + d0, s0);
                            uint32_t best = 0xFFFFFFFFu;
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                const uint32_t s = __vadd2(s0[k], gsum[k]);
                                const int d = d0 + 2 * k;
                                if (d < D && d <= j) best = min(best, ((s & 0xFFFFu) << 16) | (uint32_t)d);
                                if (d + 1 < D && d + 1 <= j) best = min(best, (s & 0xFFFF0000u) | (uint32_t)(d + 1));
                            }
                            best = __reduce_min_sync(FULL, best);
                            if (lane == 0) {
                                const uint32_t disp = best & 0xFFFFu;
                                if (a.disp) a.disp[pix] = (uint16_t)disp;
                                if (a.out) {
                                    const int oi = i - a.dc, oj = j - a.dc;
                                    if (oi >= 0 && oi < a.h && oj >= 0 && oj < a.w)
                                        a.out[(size_t)oi * a.w + oj] = (uint16_t)min(disp * 255u, 0xFFFFu);
                                }
                            }
                        }
                    }
                    cp_wait<0>();
                }
            } else if (wi == R && has_fetcher) {
                // ======================================================= fetcher: previous group's last row -> ring 0
                const uint16_t *src = a.bnd + (size_t)(grp - 1) * W * rec;
                const unsigned *prog = a.progress + (grp - 1);
                const int nch = rec / 8; // 16-byte chunks per record
                unsigned seen = 0;
                for (int x = 0; x < W; x++) {
                    const int s = x & (kK - 1);
                    if (x >= kK) mbar_wait<false>(empty_bar(0, s), ((x / kK) - 1) & 1, a);
                    if (seen < (unsigned)x + 1u) {
                        for (unsigned n = 0;; n++) {
                            const unsigned v = ld_acquire(prog);
                            if (v >= (unsigned)x + 1u) { seen = v; break; }
                            if (ld_acquire(a.err) != kErrNone || n > a.spin_limit) {
                                atomicCAS(a.err, kErrNone, kErrTimeout);
                                seen = 0xFFFFFFFFu;
                                break;
                            }
                            __nanosleep(64);
                        }
                    }
                    const uint4 *g4 = reinterpret_cast<const uint4 *>(src + (size_t)x * rec);
                    uint4 *s4 = reinterpret_cast<uint4 *>(ring_slot(0, s));
                    for (int k = lane; k < nch; k += 32) s4[k] = __ldcg(g4 + k);
                    mbar_arrive_local(full_bar(0, s));
                }
            } else if (wi == R + 1 && has_publisher) {
                // ======================================================= publisher: this group's last row -> global
                uint16_t *dst = a.bnd + (size_t)grp * W * rec;
                const int nch = rec / 8;
                for (int x = 0; x < W; x++) {
                    const int s = x & (kK - 1);
                    mbar_wait<false>(full_bar(R, s), (x / kK) & 1, a);
                    const uint4 *s4 = reinterpret_cast<const uint4 *>(ring_slot(R, s));
                    uint4 *g4 = reinterpret_cast<uint4 *>(dst + (size_t)x * rec);
                    for (int k = lane; k < nch; k += 32) g4[k] = s4[k];
                    mbar_arrive_local(empty_bar(R, s));
                    if ((x & 7) == 7 || x == W - 1) {
                        __threadfence();
                        __syncwarp();
                        if (lane == 0) st_release(a.progress + grp, (unsigned)(x + 1));
                    }
                }
            }
        }
        cluster_sync();
    }
}

template <int DPL>
void set_attrs(int optin) {
    cudaFuncSetAttribute(sgm_kernel<DPL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaFuncSetAttribute(sgm_kernel<DPL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

template <int DPL>
const void *kernel_ptr(int pass) {
    return pass ? (const void *)sgm_kernel<DPL, 1> : (const void *)sgm_kernel<DPL, 0>;
}
const void *kernel_for(int dpl, int pass) {
    switch (dpl) {
    case 2: return kernel_ptr<2>(pass);
    case 4: return kernel_ptr<4>(pass);
    case 6: return kernel_ptr<6>(pass);
    case 8: return kernel_ptr<8>(pass);
    case 12: return kernel_ptr<12>(pass);
    case 16: return kernel_ptr<16>(pass);
    default: return nullptr;
    }
}

int max_active_clusters(const void *fn, int cs, int threads, size_t smem) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cs * 64);
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

} // namespace

void init_sgm_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    set_attrs<2>(optin); set_attrs<4>(optin); set_attrs<6>(optin);
    set_attrs<8>(optin); set_attrs<12>(optin); set_attrs<16>(optin);
    cudaGetLastError();
}

SgmPlan sgm_plan(const Geom &g, int device, int force_R, int force_cs) {
    SgmPlan best{};
    int optin = 227 * 1024, sms = 152;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaGetLastError();
    int rmax = g.dpl >= 12 ? 8 : 16;
    while (rmax > 1 && sgm_smem(rmax, g.dp, 1).total > (size_t)optin) rmax--;
    const void *fn = kernel_for(g.dpl, 1);
    if (!fn) return best;
    for (int cs : {8, 4, 2, 1}) {
        if (force_cs && cs != force_cs) continue;
        // co-resident clusters depend on the CTA size, which depends on R: iterate to a fixed point
        int R = std::max(1, std::min(rmax, (g.Hp + sms - 1) / sms));
        if (force_R) R = std::max(1, std::min(rmax, force_R));
        int clusters = 0;
        for (int it = 0; it < 4; it++) {
            clusters = max_active_clusters(fn, cs, (R + 2) * 32, sgm_smem(R, g.dp, 1).total);
            if (clusters < 1 || force_R) break;
            const int want = (g.Hp + clusters * cs - 1) / (clusters * cs);
            const int nr = std::max(1, std::min(rmax, want));
            if (nr == R) break;
            R = nr;
        }
        if (clusters < 1) continue;
        SgmPlan p{};
        p.R = R;
        p.cs = cs;
        p.nbands = (g.Hp + R - 1) / R;
        p.ngroups = (p.nbands + cs - 1) / cs;
        p.nclusters = std::min(p.ngroups, clusters);
        // prefer fewer rows per CTA (shorter steps), then larger clusters (fewer global hand-offs)
        if (best.R == 0 || p.R < best.R) best = p;
    }
    return best;
}

size_t sgm_bnd_bytes(const Geom &g, const SgmPlan &p) {
    return (size_t)std::max(p.ngroups, 1) * g.Wp * rec_u16(g.dp) * sizeof(uint16_t);
}

cudaError_t launch_sgm_pass(const Geom &g, const SgmPlan &p, SgmArgs a, int pass, cudaStream_t st) {
    if (p.R < 1) return cudaErrorInvalidConfiguration;
    a.R = p.R;
    a.cs = p.cs;
    a.nbands = p.nbands;
    a.ngroups = p.ngroups;
    const void *fn = kernel_for(g.dpl, pass);
    if (!fn) return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(a.progress, 0, (size_t)p.ngroups * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(p.nclusters * p.cs);
    cfg.blockDim = dim3((p.R + 2) * 32);
    cfg.dynamicSmemBytes = sgm_smem(p.R, g.dp, pass).total;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = p.cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    void *args[] = {(void *)&a};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

} // namespace sister
