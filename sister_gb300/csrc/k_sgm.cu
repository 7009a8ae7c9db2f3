// 8-path semi-global aggregation (sgm.cpp:26-455, called as sgm(.., 7, 17, 8) at
// SisterMultiviewDisparities.hpp:280) fused with the final winner-take-all (hpp:283), crop and *255 (hpp:111-118).
//
// The reference runs two raster passes; each pass updates four paths per pixel:
//   r0 from (i, j-dj), r1 from (i-di, j-dj), r2 from (i-di, j), r3 from (i-di, j+dj)
// with P1 = 7 and a constant P2 = 100 (adaptP2 with alpha = 0, sgm.cpp:15-22, :34-35). In pass
// coordinates (row r, column q; pass 1 mirrors both axes) a path value at (r, q) depends on its own
// predecessor only: r0 on (r, q-1), r1 on (r-1, q-1), r2 on (r-1, q), r3 on (r-1, q+1). The paths are
// coupled only through the per-pixel sum.
//
// The two passes are independent until their sums meet, so one persistent launch runs the bands of both
// interleaved (work item k: pass k & 1, band k >> 1); each pass stores its 4-path sum and a final
// memory-bound kernel adds the two sums and takes the winner-take-all. While the bands of one pass wait
// on the wavefront above them, the other pass's bands keep the SMs busy.
//
// Work decomposition (one CTA = a band of R image rows, persistent over work items)
//   * four "path warps" per row, one per path, each sweeping q = 0..W-1 with 32 lanes x DPL disparities.
//     The row-to-row dependency chain (r3 trails the row above by one column) therefore costs one path
//     update per hop instead of four;
//   * the r0 warp of a row also owns the row's sum: it gathers r1, r2, r3 of each pixel from the other
//     three warps, adds r0, and stores the pass's 4-path sum;
//   * the r1, r2, r3 states of a row go to a KP-slot ring with one full barrier per slot (all three path
//     warps arrive) and one empty barrier per slot (the row's r0 warp and the next row's three path warps
//     arrive); producers check the empty barriers once per KP/2 pixels;
//   * data from global memory arrives by bulk copies (TMA). A warp completes about one asynchronous copy
//     per global-memory round trip however large it is (measured on GB300: ~500-750 cycles per copy for
//     anything from 512 B to 16 KB), so every stream is copied in batches: the cost rows of FB
//     consecutive pixels per copy into a two-group ring per row shared by the row's four warps, one group
//     ahead;
//   * the last row of a band is handed to the next band through global memory: a collector warp copies
//     it into a staging ring (so the row never waits on global memory), a writer warp stores the records
//     and, at the end of every hand-off batch (2, 2, 4 pixels, then FB at a time), fences and releases a
//     progress counter. A fetcher warp of the next band polls that counter and bulk-copies each batch of
//     records into a ring of 2*FB slots for its first row, so a band starts two pixels after the one above. In the
//     first band the fetcher feeds the first line's cost rows to that line's path warps instead (they
//     need no input), so the slow 8-bit-truncated r0 recurrence of the first line paces no other row.
//     Compute warps never fence or poll global memory.
// Arithmetic is packed u16x2: minima with __vminu2, additions and subtractions as plain 32-bit IADDs, which
// equal packed u16x2 ones whenever no half carries or borrows. That holds on the recurrence: a path value is
// C + (m - minLp) with minLp <= m <= minLp + 100, so real entries stay below 1021 + 100 and "infinite"
// entries (missing columns, disparities >= dc, stored as 0x7FFF) below 0x8064 (+7 < 0x10000); m - minLp
// never borrows since every half of m is >= minLp. Only the 4-path sum of an infinite pair can exceed 16
// bits; dc is a multiple of 8, so both halves of a pair are real or both infinite, and that carry stays
// inside a pair whose sums are never read (the final minimum masks d >= dc).
// Every wait is bounded: on expiry the device error flag is raised and the kernel finishes.
#include "sister_internal.h"

#include <algorithm>

namespace sister {

constexpr int kHelpers = 3;      // fetcher, collector, writer warps
constexpr int kRowsMax = 7;      // rows per band for DPL <= 8: 4*7+3 = 31 warps
constexpr int kRowsMaxWide = 6;  // rows per band for DPL >= 12: 27 warps (register file)
constexpr int kKS = 8;           // staging-ring slots of the band's last row
// pixels per batched copy: cost group of a row, and records (or first-line cost rows) per fetch
__host__ __device__ constexpr int batch_px(int dp) { return dp >= 384 ? 4 : 8; }
// path-ring slots (power of two; producers check the empty barriers every half ring)
__host__ __device__ constexpr int path_slots(int dp) { return dp >= 384 ? 4 : 8; }

// global hand-off record between bands: r1 | r2 | r3 (dp u16 each) | minima m1 m2 m3 (+5 pad)
__host__ __device__ inline int rec_u16(int dp) { return 3 * dp + 8; }
// one path state in a ring slot: state (dp u16) | minimum (+7 pad)
__host__ __device__ inline int pslot_u16(int dp) { return dp + 8; }

struct SgmSmem {
    size_t bars, prings, inring, stage, cring, total;
    int nbar;
};
// barrier layout (8 bytes each; FB = batch_px(dp), KI = 2*FB, KP = path_slots(dp)):
//   path ring of row w, slot s: full at 2*(w*KP + s), empty at +1
//   incoming ring: batch full barriers [2] at in_base, per-slot empty barriers [KI] after them
//   staging ring slot s: full at st_base + 2s, empty at +1;  cost group g (0, 1) of row w: c_base + 2w + g
__host__ __device__ inline SgmSmem sgm_smem(int R, int dp) {
    SgmSmem L{};
    const int FB = batch_px(dp), KI = 2 * FB, KP = path_slots(dp);
    L.nbar = R * KP * 2 + 2 + KI + kKS * 2 + R * 2;
    size_t o = 0;
    L.bars = o;
    o += (size_t)L.nbar * 8;
    o = (o + 127) & ~(size_t)127;
    L.prings = o;
    o += (size_t)R * KP * 3 * pslot_u16(dp) * 2;
    L.inring = o;
    o += (size_t)KI * rec_u16(dp) * 2;
    L.stage = o;
    o += (size_t)kKS * rec_u16(dp) * 2;
    o = (o + 127) & ~(size_t)127;
    L.cring = o;
    o += (size_t)R * 2 * FB * dp * 2;
    L.total = o;
    return L;
}

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t INF2 = 0x7FFF7FFFu;

// ---------------------------------------------------------------- PTX helpers
__device__ __forceinline__ uint32_t sptr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void mbar_init(uint32_t a, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint32_t a) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
                 : "memory");
}
// 1D bulk copy global -> shared of this CTA, completion counted on mbarrier `bar`
// (both addresses 16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// non-blocking test of the phase of parity `par`
__device__ __forceinline__ bool mbar_test(uint32_t a, uint32_t par) {
    uint32_t ok;
    asm volatile("{ .reg .pred p; mbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2; "
                 "selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok)
                 : "r"(a), "r"(par)
                 : "memory");
    return ok != 0;
}
// blocking test: the warp sleeps until the phase completes or about `ns` nanoseconds pass, so waiting
// warps take no issue slots from the warps doing the arithmetic
__device__ __forceinline__ bool mbar_sleep(uint32_t a, uint32_t par, uint32_t ns) {
    uint32_t ok;
    asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2, %3; "
                 "selp.u32 %0, 1, 0, p; }"
                 : "=r"(ok)
                 : "r"(a), "r"(par), "r"(ns)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
constexpr uint32_t kSleepNs = 20000; // suspend hint of one blocking test
constexpr unsigned kCheckEvery = 64; // blocking tests between looks at the error flag and the clock (a
                                     // global load costs a memory round trip, which would delay every
                                     // hand-off that just missed its first test)
// Bounded wait for the phase of parity `par`: after g.wait_limit_us microseconds, or once another warp has
// raised the device error flag, the flag is raised and the caller proceeds (the host then reports
// SISTER_ETIMEOUT), so no wait can hang the GPU.
__device__ __forceinline__ void mbar_wait(uint32_t a, uint32_t par, const SgmLaunch &g) {
    if (mbar_test(a, par)) return;
    unsigned long long t0 = 0;
    for (unsigned n = 0;; n++) {
        if (mbar_sleep(a, par, kSleepNs)) return;
        if (n % kCheckEvery == kCheckEvery - 1) {
            const unsigned long long t = global_ns();
            if (t0 == 0) t0 = t;
            if (ld_relaxed(g.err) != kErrNone || t - t0 > 1000ull * g.wait_limit_us) {
                atomicCAS(g.err, kErrNone, kErrTimeout);
                return;
            }
        }
    }
}
// Wait for the phase of parity `par` with a time limit only (no early exit on the error flag): used to
// drain bulk copies still in flight before barriers are re-initialised or the CTA exits.
__device__ __forceinline__ void mbar_drain(uint32_t a, uint32_t par, unsigned limit_us) {
    if (mbar_test(a, par)) return;
    const unsigned long long t0 = global_ns();
    while (!mbar_sleep(a, par, kSleepNs) && global_ns() - t0 <= 1000ull * limit_us) {
    }
}
// order this thread's generic-proxy view of global memory (acquired records) before its bulk copies
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;" ::: "memory");
}

// NP consecutive 32-bit words (2*NP u16) from / to shared or global memory, widest aligned accesses
template <int NP>
__device__ __forceinline__ void ldw(const uint16_t *p, uint32_t (&o)[NP]) {
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
__device__ __forceinline__ void stw(uint16_t *p, const uint32_t (&v)[NP]) {
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
        const uint32_t t = __vminu2(xprev, x) + 0x00070007u;
        const uint32_t m = __vminu2(t, __vminu2(P[k], p2));
        const uint32_t v = C[k] + m - m2;
        Ln[k] = v;
        mn = __vminu2(mn, v);
        xprev = x;
    }
    return hmin(mn);
}

// ---------------------------------------------------------------- the kernel
template <int DPL>
__global__ void __launch_bounds__((4 * (DPL >= 12 ? kRowsMaxWide : kRowsMax) + kHelpers) * 32, 1)
    sgm_kernel(const SgmLaunch a) {
    constexpr int NP = DPL / 2;
    constexpr int KP = path_slots(32 * DPL), EB = KP / 2;
    constexpr int FB = batch_px(32 * DPL); // pixels per batched copy
    constexpr int KI = 2 * FB;             // incoming-ring slots (two batches)
    extern __shared__ __align__(128) unsigned char smem[];
    const int R = a.R, dp = a.dp;
    int W = 0, H = 0; // geometry of the current work item's rig
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int d0 = lane * DPL;
    const int rec = rec_u16(dp), ps = pslot_u16(dp);
    const SgmSmem L = sgm_smem(R, dp);
    const uint32_t bars = sptr(smem + L.bars);
    auto pfull = [&](int w, int s) { return bars + 16u * (uint32_t)(w * KP + s); };
    auto pempty = [&](int w, int s) { return bars + 16u * (uint32_t)(w * KP + s) + 8u; };
    const uint32_t in_base = bars + 16u * (uint32_t)(R * KP);
    auto infull = [&](int b) { return in_base + 8u * (uint32_t)(b & 1); };         // batch b
    auto inempty = [&](int x) { return in_base + 16u + 8u * (uint32_t)(x & (KI - 1)); }; // pixel x's slot
    const uint32_t st_base = in_base + 16u + 8u * (uint32_t)KI;
    auto sfull = [&](int s) { return st_base + 16u * (uint32_t)s; };
    auto sempty = [&](int s) { return st_base + 16u * (uint32_t)s + 8u; };
    const uint32_t c_base = st_base + 16u * (uint32_t)kKS;
    auto cfull = [&](int w, int g) { return c_base + 8u * (uint32_t)(w * 2 + (g & 1)); };
    uint16_t *prings = reinterpret_cast<uint16_t *>(smem + L.prings);
    // state of path p (1..3) of row w in slot s
    auto pslot = [&](int w, int p, int s) { return prings + (size_t)((w * KP + s) * 3 + (p - 1)) * ps; };
    uint16_t *inring = reinterpret_cast<uint16_t *>(smem + L.inring);
    uint16_t *stage = reinterpret_cast<uint16_t *>(smem + L.stage);
    uint16_t *cring = reinterpret_cast<uint16_t *>(smem + L.cring);

    uint32_t padm[NP]; // halves holding disparities >= dc of the current rig are infinite
    int pass = 0;      // pass of the current work item: 0 top-down left-to-right, 1 mirrored
    // A batch b of FB pixels (q = FB*b ...) covers nb = min(FB, W - FB*b) pixels; in memory (columns j)
    // they are contiguous, ascending in pass 0 and descending in pass 1. offset of pixel q in its batch:
    auto boff = [&](int q) {
        const int t = q % FB;
        return pass ? (min(FB, W - (q - t)) - 1 - t) : t;
    };
    // first column (lowest j) of batch b, and its pixel count
    auto bj0 = [&](int b) { return pass ? max(0, W - FB * (b + 1)) : FB * b; };
    auto bn = [&](int b) { return min(FB, W - FB * b); };
    // Hand-off batches of the incoming stream (previous band's records, or the first line's cost rows) start
    // small so that a band can begin two pixels after the band above: pixels [0,2) [2,4) then doubling up to
    // FB, then FB at a time (FB = 8: starts 0 2 4 8 16 24 ...). No batch wraps around the ring.
    constexpr int NPF = (FB == 8) ? 3 : 2; // batches before the first full one
    auto hstart = [&](int b) { return b < NPF ? (b == 0 ? 0 : (1 << b)) : FB * (b - NPF + 1); };
    auto hend = [&](int b) { return min(W, hstart(b + 1)); };
    auto hbatch = [&](int x) { return x < FB ? (x < 2 ? 0 : 31 - __clz(x)) : x / FB + NPF - 1; };

    const int role = wi / R; // 0: r0 + sum, 1..3: paths r1..r3, then fetcher, collector, writer
    const int w = wi % R;    // row within the band (compute warps)
    bool first_band = true;
    for (int item = blockIdx.x; item < a.nitems; item += gridDim.x) {
        int band;
        SgmRig rg;
        if (a.items) {
            const uint32_t v = a.items[item];
            rg = a.rigs[v >> 24];
            band = (int)((v >> 1) & 0x7FFFFFu);
            pass = (int)(v & 1u);
        } else {
            rg = a.rig0;
            band = item >> 1;
            pass = item & 1;
        }
        W = rg.W;
        H = rg.H;
#pragma unroll
        for (int k = 0; k < NP; k++)
            padm[k] = ((d0 + 2 * k < rg.D) ? 0u : 0x0000FFFFu) | ((d0 + 2 * k + 1 < rg.D) ? 0u : 0xFFFF0000u);
        const int nhb = hbatch(W - 1) + 1;
        const int nbat = (W + FB - 1) / FB;
        const uint16_t *cost = rg.cost;
        uint16_t *sum = pass ? rg.sum1 : rg.sum0;
        uint16_t *bnd = rg.bnd + (size_t)pass * rg.nbands * W * rec;
        unsigned *progress = rg.progress + (size_t)pass * rg.nbands;
        const int row0 = band * R;
        const int rows = min(R, H - row0);
        const bool publish = rows == R && band + 1 < rg.nbands;
        if (threadIdx.x == 0) {
            if (!first_band)
                for (int k = 0; k < L.nbar; k++) mbar_inval(bars + 8u * k);
            for (int wr = 0; wr < R; wr++) {
                // consumers of a row's slots: its r0 warp (32; not on the first line of the pass), plus the next
                // row's three path warps (96) or, for the band's last row when another band follows, the
                // collector (32)
                const unsigned cons = ((row0 + wr == 0) ? 0u : 32u) +
                                      ((wr + 1 < rows) ? 96u : (wr == R - 1 && publish) ? 32u : 0u);
                for (int s = 0; s < KP; s++) {
                    mbar_init(pfull(wr, s), 96);
                    mbar_init(pempty(wr, s), cons > 0 ? cons : 1);
                }
                for (int g = 0; g < 2; g++) mbar_init(cfull(wr, g), 1); // r0's arrive.expect_tx + bytes
            }
            for (int b = 0; b < 2; b++) mbar_init(infull(b), 1);    // fetcher's arrive.expect_tx + bytes
            for (int x = 0; x < KI; x++) mbar_init(inempty(x), 96); // the first row's r1, r2, r3 warps
            for (int s = 0; s < kKS; s++) {
                mbar_init(sfull(s), 32);  // collector
                mbar_init(sempty(s), 32); // writer
            }
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        }
        first_band = false;
        __syncthreads();

        if (role < 4 && w < rows) {
            const int r = row0 + w;
            const int i = pass ? (H - 1 - r) : r;
            const bool first_line = (r == 0);
            const size_t rowbase = (size_t)i * W;
            uint16_t *myc = cring + (size_t)w * 2 * FB * dp;
            // position of pixel q in the row's cost ring: group (q/FB) & 1
            auto cidx = [&](int q) { return (size_t)((((q / FB) & 1) * FB) + boff(q)) * dp; };
            if (role == 0) {
                // ================================================= r0 warp: cost prefetch, r0, sum
                auto prefetch = [&](int b) {
                    if (lane == 0 && b < nbat) {
                        const uint32_t bytes = (uint32_t)(bn(b) * dp * 2);
                        const size_t pix = rowbase + bj0(b);
                        mbar_expect_tx(cfull(w, b), bytes);
                        bulk_g2s(sptr(myc + (size_t)(b & 1) * FB * dp), cost + pix * dp, bytes, cfull(w, b));
                    }
                };
                prefetch(0);
                // r0 restarts every row from Lp = 0, minLp = 0 (sgm.cpp:215-216)
                uint32_t r0[NP];
                uint32_t r0min = 0;
#pragma unroll
                for (int k = 0; k < NP; k++) r0[k] = INF2 & padm[k];
                for (int q = 0; q < W; q++) {
                    if (q % FB == 0) {
                        // group q/FB + 1 reuses the slots of group q/FB - 1, which every warp of the row has
                        // finished: this warp gathered the path states of its last pixel (on the first line
                        // this warp is the ring's only reader)
                        prefetch(q / FB + 1);
                        mbar_wait(cfull(w, q / FB), (q / FB / 2) & 1, a);
                    }
                    const size_t ci = cidx(q);
                    uint32_t c[NP];
                    ldw<NP>(myc + ci + d0, c);
                    uint32_t g[NP];
                    if (first_line) {
                        // First line (sgm.cpp:103-207): C' = (C == 255 ? 0 : C); r0 starts as C' and then runs the
                        // recurrence in int32 truncated to 8 bits (saturate_cast<uint16>(uint8), types.h:28);
                        // the sum receives r0 alone. r1..r3 of the first line only feed the row below.
                        uint32_t cp[NP];
#pragma unroll
                        for (int k = 0; k < NP; k++) cp[k] = c[k] & ~__vcmpeq2(c[k], 0x00FF00FFu);
                        uint32_t mnv = 0xFFFFFFFFu;
                        if (q == 0) {
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                g[k] = cp[k];
                                mnv = __vminu2(mnv, cp[k]);
                            }
                        } else {
                            uint32_t tmp[NP];
                            path_step<NP>(r0, r0min, cp, tmp, lane);
#pragma unroll
                            for (int k = 0; k < NP; k++) {
                                g[k] = (tmp[k] & 0x00FF00FFu & ~padm[k]) | (INF2 & padm[k]);
                                mnv = __vminu2(mnv, g[k]);
                            }
                        }
#pragma unroll
                        for (int k = 0; k < NP; k++) r0[k] = g[k];
                        r0min = __reduce_min_sync(FULL, hmin(mnv));
                    } else {
                        uint32_t n0[NP];
                        const uint32_t mn = path_step<NP>(r0, r0min, c, n0, lane);
                        r0min = __reduce_min_sync(FULL, mn);
                        const int s = q & (KP - 1);
                        uint32_t v1[NP], v2[NP], v3[NP];
                        mbar_wait(pfull(w, s), (q / KP) & 1, a);
                        ldw<NP>(pslot(w, 1, s) + d0, v1);
                        ldw<NP>(pslot(w, 2, s) + d0, v2);
                        ldw<NP>(pslot(w, 3, s) + d0, v3);
                        mbar_arrive(pempty(w, s));
#pragma unroll
                        for (int k = 0; k < NP; k++) {
                            r0[k] = n0[k];
                            g[k] = n0[k] + v1[k] + v2[k] + v3[k];
                        }
                    }
                    // the pass's sum: first line r0 alone (sgm.cpp:132, :187), else r0+r1+r2+r3 (:386-391); u16
                    // arithmetic never saturates or wraps for real disparities
                    stw<NP>(sum + (rowbase + (pass ? (W - 1 - q) : q)) * dp + d0, g);
                }
                // every copy this warp issued has been waited for; after a timeout a wait may have returned
                // early, so make sure none is still in flight before the barriers are reused
                if (lane == 0)
                    for (int b = max(0, nbat - 2); b < nbat; b++) mbar_drain(cfull(w, b), (b / 2) & 1, a.wait_limit_us);
            } else {
                // ================================================= path warp p = role (1: r1, 2: r2, 3: r3)
                const int p = role;
                // input: the same path of the row above -- the ring of row w-1, or the incoming ring for w == 0
                const bool from_in = (w == 0);
                for (int q = 0; q < W; q++) {
                    uint32_t c[NP];
                    if (first_line) {
                        // the first line's path warps take their cost rows from the fetcher's batches (incoming
                        // ring, row of pixel q at position q % KI, batches stored in memory order), not from the
                        // r0 warp's cost ring
                        const int hb = hbatch(q), hs = hstart(hb), he = hend(hb);
                        if (q == hs) mbar_wait(infull(hb), (hb / 2) & 1, a);
                        ldw<NP>(inring + (size_t)(hs % KI + (pass ? he - 1 - q : q - hs)) * dp + d0, c);
                        mbar_arrive(inempty(q));
                    } else {
                        if (q % FB == 0) mbar_wait(cfull(w, q / FB), (q / FB / 2) & 1, a);
                        ldw<NP>(myc + cidx(q) + d0, c);
                    }
                    uint32_t out[NP];
                    uint32_t mn;
                    if (first_line) {
                        // first line: r1..r3 take C' with minimum min(C') (sgm.cpp:112-114, :149-151, :192-194)
                        uint32_t mnv = 0xFFFFFFFFu;
#pragma unroll
                        for (int k = 0; k < NP; k++) {
                            out[k] = c[k] & ~__vcmpeq2(c[k], 0x00FF00FFu);
                            mnv = __vminu2(mnv, out[k]);
                        }
                        mn = hmin(mnv);
                    } else {
                        // r3 reads column q+1 of the row above and never column 0: release that slot unread
                        if (p == 3 && q == 0) mbar_arrive(from_in ? inempty(0) : pempty(w - 1, 0));
                        // predecessor column: q-1 (r1), q (r2), q+1 (r3); outside the image: inf with min 0
                        const int x = q + p - 2;
                        uint32_t P[NP];
                        uint32_t mp = 0;
                        if (x >= 0 && x < W) {
                            if (from_in) {
                                // records arrive in batches; consumers take them in order, so a wait at the first
                                // record of each batch (or the first one this warp reads) suffices
                                const int hb = hbatch(x);
                                if (x == hstart(hb) || x == (p == 3 ? 1 : 0)) mbar_wait(infull(hb), (hb / 2) & 1, a);
                                const uint16_t *src = inring + (size_t)(x & (KI - 1)) * rec;
                                ldw<NP>(src + (size_t)(p - 1) * dp + d0, P);
                                mp = src[3 * dp + p - 1];
                                mbar_arrive(inempty(x));
                            } else {
                                const int s = x & (KP - 1);
                                mbar_wait(pfull(w - 1, s), (x / KP) & 1, a);
                                const uint16_t *src = pslot(w - 1, p, s);
                                ldw<NP>(src + d0, P);
                                mp = src[dp];
                                mbar_arrive(pempty(w - 1, s));
                            }
                        } else {
#pragma unroll
                            for (int k = 0; k < NP; k++) P[k] = INF2;
                        }
                        mn = path_step<NP>(P, mp, c, out, lane);
                    }
                    const uint32_t m = __reduce_min_sync(FULL, mn);
                    // slots q .. q+EB-1 last held pixels q-KP .. q-KP+EB-1; every consumer releases in pixel
                    // order, so the release of the last of them covers all
                    if (q >= KP && (q & (EB - 1)) == 0) {
                        const int y = q - KP + EB - 1;
                        mbar_wait(pempty(w, y & (KP - 1)), (y / KP) & 1, a);
                    }
                    const int s = q & (KP - 1);
                    uint16_t *dst = pslot(w, p, s);
                    stw<NP>(dst + d0, out);
                    if (lane == 0) dst[dp] = (uint16_t)m;
                    mbar_arrive(pfull(w, s));
                }
            }
        } else if (wi == 4 * R) {
            // ===================================================== fetcher: batches of FB pixels -> inring
            // band 0: the first line's cost rows; later bands: the previous band's last-row records
            if (lane == 0) {
                const uint16_t *src = bnd + (size_t)(band > 0 ? band - 1 : 0) * W * rec;
                const unsigned *prog = progress + (band > 0 ? band - 1 : 0);
                const size_t rowbase0 = (size_t)(pass ? H - 1 : 0) * W;
                unsigned seen = 0;
                for (int b = 0; b < nhb; b++) {
                    const int hs = hstart(b), he = hend(b), nb = he - hs;
                    // before reusing barrier b & 1 every reader must be past batch b-2, and the ring slots of
                    // pixels hs..he-1 must be free (they last held pixels hs-KI..he-1-KI); readers release in
                    // pixel order, so waiting for the later of the two last pixels covers both
                    const int y = max(b >= 2 ? hend(b - 2) - 1 : -1, he - 1 - KI);
                    if (y >= 0) mbar_wait(inempty(y), (y / KI) & 1, a);
                    if (band == 0) {
                        const uint32_t bytes = (uint32_t)(nb * dp * 2);
                        mbar_expect_tx(infull(b), bytes);
                        bulk_g2s(sptr(inring + (size_t)(hs % KI) * dp), cost + (rowbase0 + (pass ? W - he : hs)) * dp,
                                 bytes, infull(b));
                        continue;
                    }
                    uint16_t *dst = inring + (size_t)(hs % KI) * rec;
                    const unsigned need = (unsigned)he;
                    if (seen < need) {
                        const unsigned long long t0 = global_ns();
                        for (unsigned n = 0;; n++) {
                            const unsigned v = ld_acquire(prog);
                            if (v >= need) {
                                seen = v;
                                break;
                            }
                            if (n % kCheckEvery == kCheckEvery - 1 &&
                                (ld_relaxed(a.err) != kErrNone || global_ns() - t0 > 1000ull * a.wait_limit_us)) {
                                atomicCAS(a.err, kErrNone, kErrTimeout);
                                seen = 0xFFFFFFFFu;
                                break;
                            }
                        }
                        fence_proxy_async_global();
                    }
                    const uint32_t bytes = (uint32_t)(nb * rec * 2);
                    mbar_expect_tx(infull(b), bytes);
                    bulk_g2s(sptr(dst), src + (size_t)hs * rec, bytes, infull(b));
                }
                for (int b = max(0, nhb - 2); b < nhb; b++) mbar_drain(infull(b), (b / 2) & 1, a.wait_limit_us);
            }
        } else if (wi == 4 * R + 1 && publish) {
            // ===================================================== collector: band's last row -> staging ring
            const int wl = R - 1;
            for (int x = 0; x < W; x++) {
                const int s = x & (kKS - 1);
                if (x >= kKS) mbar_wait(sempty(s), ((x / kKS) - 1) & 1, a);
                uint16_t *sd = stage + (size_t)s * rec;
                const int ks = x & (KP - 1);
                mbar_wait(pfull(wl, ks), (x / KP) & 1, a);
                for (int p = 1; p <= 3; p++) {
                    const uint16_t *sl = pslot(wl, p, ks);
                    const uint4 *s4 = reinterpret_cast<const uint4 *>(sl);
                    uint4 *d4 = reinterpret_cast<uint4 *>(sd + (size_t)(p - 1) * dp);
                    for (int k = lane; k < dp / 8; k += 32) d4[k] = s4[k];
                    if (lane == 0) sd[3 * dp + p - 1] = sl[dp];
                }
                mbar_arrive(pempty(wl, ks));
                mbar_arrive(sfull(s));
            }
        } else if (wi == 4 * R + 2 && publish) {
            // ===================================================== writer: staging ring -> global, progress
            uint16_t *dst = bnd + (size_t)band * W * rec;
            const int nch = rec / 8; // 16-byte chunks per record
            for (int x = 0; x < W; x++) {
                const int s = x & (kKS - 1);
                mbar_wait(sfull(s), (x / kKS) & 1, a);
                const uint4 *s4 = reinterpret_cast<const uint4 *>(stage + (size_t)s * rec);
                uint4 *g4 = reinterpret_cast<uint4 *>(dst + (size_t)x * rec);
                for (int k = lane; k < nch; k += 32) g4[k] = s4[k];
                mbar_arrive(sempty(s));
                // releases at the end of every hand-off batch (the fetcher copies whole batches)
                if (x + 1 == hend(hbatch(x))) {
                    __threadfence();
                    __syncwarp();
                    if (lane == 0) st_release(progress + band, (unsigned)(x + 1));
                }
            }
        }
        __syncthreads();
    }
}

// Sum of the two passes' sums and the final WTALeft (hpp:283, postprocess.cpp:74-185): the lowest
// d <= min(j, dc-1) of S0 + S1 (pass 1 adds its sum to pass 0's, saturating at sgm.cpp:390 -- real sums
// stay below 2 * 4 * 1121, so nothing saturates), then crop and *255 (hpp:111-118). One warp per padded
// pixel, lanes over d; memory-bound (reads both sum volumes once).
template <int DPL>
__global__ void __launch_bounds__(256) sgm_wta_kernel(const uint16_t *__restrict__ s0v, const uint16_t *__restrict__ s1v,
                                                      Geom g, uint16_t *__restrict__ out, uint16_t *__restrict__ disp) {
    constexpr int NP = DPL / 2;
    const int lane = threadIdx.x & 31;
    const size_t pix = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (pix >= g.plane) return;
    const int i = (int)(pix / g.Wp), j = (int)(pix % g.Wp);
    const int d0 = lane * DPL, D = g.dc;
    uint32_t s0[NP], s1[NP];
    ldw<NP>(s0v + pix * g.dp + d0, s0);
    ldw<NP>(s1v + pix * g.dp + d0, s1);
    // keys (sum << 16) | d; halves with d >= dc or d > j are forced to sum 0xFFFF (real sums are smaller)
    uint32_t best = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        const int d = d0 + 2 * k;
        uint32_t sv = s0[k] + s1[k]; // both halves of a pair are real or both infinite (dc % 8 == 0)
        if (d >= D || d > j) sv |= 0x0000FFFFu;
        if (d + 1 >= D || d + 1 > j) sv |= 0xFFFF0000u;
        best = min(best, min(__byte_perm(sv, (uint32_t)d, 0x1054), __byte_perm(sv, (uint32_t)(d + 1), 0x3254)));
    }
    best = __reduce_min_sync(FULL, best);
    if (lane == 0) {
        const uint32_t dv = best & 0xFFFFu;
        if (disp) disp[pix] = (uint16_t)dv;
        const int oi = i - g.dc, oj = j - g.dc;
        if (out && oi >= 0 && oi < g.h && oj >= 0 && oj < g.w) out[(size_t)oi * g.w + oj] = (uint16_t)min(dv * 255u, 0xFFFFu);
    }
}

const void *kernel_for(int dpl) {
    switch (dpl) {
    case 2: return (const void *)sgm_kernel<2>;
    case 4: return (const void *)sgm_kernel<4>;
    case 6: return (const void *)sgm_kernel<6>;
    case 8: return (const void *)sgm_kernel<8>;
    case 12: return (const void *)sgm_kernel<12>;
    case 16: return (const void *)sgm_kernel<16>;
    default: return nullptr;
    }
}

} // namespace

void init_sgm_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    for (int dpl : kDplChoices) cudaFuncSetAttribute(kernel_for(dpl), cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaGetLastError();
}

// largest band height whose shared-memory layout fits this device
int sgm_rows_max(int dp, int device) {
    int optin = 227 * 1024;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaGetLastError();
    int rmax = dp >= 384 ? kRowsMaxWide : kRowsMax;
    while (rmax > 1 && sgm_smem(rmax, dp).total > (size_t)optin) rmax--;
    return rmax;
}

// Rows per band: enough bands to cover the image in one wave of persistent CTAs when it fits
// (R = ceil(Hp / SMs)), else the largest band the block can hold; force_R overrides (tuning).
// ngroups counts the work items of one launch (two passes x nbands), each with a progress counter and a
// hand-off record row.
SgmPlan sgm_plan(const Geom &g, int device, int force_R, int /*force_cs: bands are never clustered*/) {
    SgmPlan p{};
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaGetLastError();
    const int rmax = sgm_rows_max(g.dp, device);
    int R = std::max(1, std::min(rmax, (g.Hp + sms - 1) / sms));
    if (force_R) R = std::max(1, std::min(rmax, force_R));
    const void *fn = kernel_for(g.dpl);
    if (!fn) return p;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (4 * R + kHelpers) * 32, sgm_smem(R, g.dp).total) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return p;
    }
    p.R = R;
    p.cs = 1;
    p.nbands = (g.Hp + R - 1) / R;
    p.ngroups = 2 * p.nbands;
    p.nclusters = std::min(p.ngroups, per_sm * sms); // persistent CTAs, all co-resident
    return p;
}

size_t sgm_bnd_bytes(const Geom &g, const SgmPlan &p) {
    return (size_t)std::max(p.ngroups, 1) * g.Wp * rec_u16(g.dp) * sizeof(uint16_t);
}

cudaError_t launch_sgm(const Geom &g, const SgmPlan &p, SgmRig rig, unsigned *err, cudaStream_t st) {
    if (p.R < 1) return cudaErrorInvalidConfiguration;
    const void *fn = kernel_for(g.dpl);
    if (!fn) return cudaErrorInvalidValue;
    rig.W = g.Wp;
    rig.H = g.Hp;
    rig.D = g.dc;
    rig.nbands = p.nbands;
    SgmLaunch a{};
    a.rig0 = rig;
    a.rigs = nullptr;
    a.items = nullptr;
    a.nitems = p.ngroups;
    a.R = p.R;
    a.dp = g.dp;
    a.err = err;
    a.wait_limit_us = 2000000; // 2 s
    cudaError_t e = cudaMemsetAsync(rig.progress, 0, (size_t)p.ngroups * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&a};
    // cooperative launch: every CTA is resident, and each work item depends only on work items of lower
    // index (the previous band of its pass), so no item waits on one that cannot run
    return cudaLaunchCooperativeKernel(fn, dim3(p.nclusters), dim3((p.R * 4 + kHelpers) * 32), args,
                                       sgm_smem(p.R, g.dp).total, st);
}

cudaError_t launch_sgm_multi(int dp, int R, const SgmRig *rigs_dev, const uint32_t *items_dev, int nitems,
                             unsigned *err, int device, cudaStream_t st) {
    const int dpl = dp / 32;
    const void *fn = kernel_for(dpl);
    if (!fn || R < 1 || nitems < 1) return cudaErrorInvalidValue;
    int sms = 152, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (4 * R + kHelpers) * 32, sgm_smem(R, dp).total) !=
            cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return cudaErrorInvalidConfiguration;
    }
    SgmLaunch a{};
    a.rigs = rigs_dev;
    a.items = items_dev;
    a.nitems = nitems;
    a.R = R;
    a.dp = dp;
    a.err = err;
    a.wait_limit_us = 2000000; // 2 s
    void *args[] = {(void *)&a};
    return cudaLaunchCooperativeKernel(fn, dim3(std::min(nitems, per_sm * sms)), dim3((R * 4 + kHelpers) * 32), args,
                                       sgm_smem(R, dp).total, st);
}

cudaError_t launch_sgm_wta(const Geom &g, const uint16_t *s0, const uint16_t *s1, uint16_t *out, uint16_t *disp,
                           cudaStream_t st) {
    const unsigned blocks = (unsigned)((g.plane + 7) / 8);
    switch (g.dpl) {
    case 2: sgm_wta_kernel<2><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    case 4: sgm_wta_kernel<4><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    case 6: sgm_wta_kernel<6><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    case 8: sgm_wta_kernel<8><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    case 12: sgm_wta_kernel<12><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    case 16: sgm_wta_kernel<16><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace sister
