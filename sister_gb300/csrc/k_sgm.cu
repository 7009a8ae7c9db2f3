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
// interleaved (work item k: pass k & 1, band k >> 1, drawn by the CTAs from a ticket); each pass stores its 4-path sum and a final
// memory-bound kernel adds the two sums and takes the winner-take-all. While the bands of one pass wait
// on the wavefront above them, the other pass's bands keep the SMs busy.
//
// Work decomposition (one CTA = a band of R image rows, persistent over work items)
//   * one warp per row sweeps q = 0..W-1 with 32 lanes x DPL disparities and updates all four paths of
//     the pixel: r0 from its own registers, r1/r2/r3 from the row above. Column x of the row above is
//     loaded once, at pixel x-1 (where r3 needs it), and its r2 and r1 states are kept in registers for
//     the next two pixels. The four updates are independent, so they overlap; the warp adds them into the
//     pass's sum itself. A row therefore trails the row above by about one pixel;
//   * every row hands its new r1|r2|r3 states and their minima (one record per pixel) to the row below
//     through a ring of kKP slots with a full and an empty barrier per slot; producers wait on the empty
//     barriers once per two pixels;
//   * data from global memory arrives by bulk copies (TMA). A warp completes about one asynchronous copy
//     per global-memory round trip however large it is (measured on GB300: ~500-750 cycles per copy for
//     anything from 512 B to 16 KB), so every stream is copied in batches: the cost rows of FB
//     consecutive pixels per copy into a two-group ring per row, one group ahead;
//   * the last row of a band is handed to the next band through global memory: its ring (kKS slots) is
//     read by a writer warp that stores the records and, at the end of every 2-pixel hand-off batch,
//     publishes its count in shared memory; a releaser warp turns the latest count into a device-scope
//     release of the band's progress counter, so the writer never waits on a device-wide fence (about a
//     microsecond each, longer than two pixel periods). A fetcher warp of the next band polls that counter
//     and bulk-copies each batch of records into a ring of 2*FB slots for its first row, so a band starts
//     two pixels after the one above. Row warps never fence or poll global memory.
// Arithmetic is packed u16x2: minima with __vminu2, additions and subtractions as plain 32-bit IADDs, which
// equal packed u16x2 ones whenever no half carries or borrows. That holds on the recurrence: a path value is
// C + (m - minLp) with minLp <= m <= minLp + 100, so real entries stay below 1021 + 100 and "infinite"
// entries (missing columns, disparities >= dc, stored as 0x7FFF) below 0x8064 (+7 < 0x10000); m - minLp
// never borrows since every half of m is >= minLp. Only the 4-path sum of an infinite pair can exceed 16
// bits; dc is a multiple of 8, so both halves of a pair are real or both infinite, and that carry stays
// inside a pair whose sums are never read (the final minimum masks d >= dc).
// Every wait is bounded: on expiry the device error flag is raised and the kernel finishes.
#include "sister_internal.h"
#include "ptx_sync.h"
#include "tuned_gb300.h"

#include <algorithm>
#include <cstdlib>
#include <vector>

namespace sister {

constexpr int kHelpers = 3; // fetcher, writer and releaser warps
constexpr int kKP = 4;      // ring slots of a row read by the row below
constexpr int kKS = 8;      // ring slots of the band's last row, read by the writer
constexpr int kBndRows = 2; // global hand-off rows per pass (a power of two), reused by every other band
// most rows per band (one warp each) by d-stride; shared memory may allow fewer
__host__ __device__ constexpr int rows_cap(int dp) { return dp <= 256 ? 14 : 12; }
// Pixels per batched copy (cost group of a row, and records per fetch) by d-stride and band height. At d-stride 512
// bands above 9 rows fit in shared memory only with cost groups of 2 pixels; those run their own instantiation
// (its launch bound for 12 row warps), which at 4096x3000/512 and 11 rows takes the aggregation from 32.5 to 30.5
// ms, while smaller rigs of that d-stride stay fastest at 9 rows in groups of 4 (1280x960/512: 8.09 against 8.22).
__host__ __device__ constexpr int batch_px(int dp, int R) { return dp >= 512 ? (R > 9 ? 2 : 4) : dp >= 384 ? 4 : 8; }
// most rows per band of the instantiation with cost groups of FB pixels
__host__ __device__ constexpr int rows_cap_fb(int dp, int FB) { return dp >= 512 && FB == 4 ? 9 : rows_cap(dp); }
// pixels per hand-off batch between bands (batches of 2 measured fastest once the device-wide release moved off
// the writer: 4.48 ms against 4.61 for 4 and 4.54 for 8 on 1920x1080/256), and the number of such batches the
// incoming ring (2 * batch_px slots) holds, each with its own full barrier
__host__ __device__ constexpr int hand_px(int) { return 2; }
__host__ __device__ constexpr int in_batches(int dp, int R) { return 2 * batch_px(dp, R) / hand_px(dp); }

// one pixel's record, in ring slots and in the global hand-off rows alike: r1 | r2 | r3 (dp u16 each) |
// minima m1 m2 m3, each as a u32 pair (m, m) so that it feeds the packed arithmetic directly (+2 pad)
__host__ __device__ inline int rec_u16(int dp) { return 3 * dp + 8; }

struct SgmSmem {
    size_t bars, rings, inring, cring, total;
    int nbar, nslot;
};
// ring slots: row w < R-1 owns slots [w*kKP, w*kKP + kKP), row R-1 owns [(R-1)*kKP, (R-1)*kKP + kKS)
// barriers (8 bytes each; FB = batch_px(dp, R), KI = 2*FB): slot k full at 2k, empty at 2k+1; then the incoming
// ring's batch full barriers [in_batches] and per-slot empty barriers [KI]; then cost group g (0, 1) of row w at
// 2w + g
__host__ __device__ inline SgmSmem sgm_smem_fb(int R, int dp, int FB) {
    SgmSmem L{};
    const int KI = 2 * FB;
    L.nslot = (R - 1) * kKP + kKS;
    L.nbar = 2 * L.nslot + KI / hand_px(dp) + KI + 2 * R;
    size_t o = 0;
    L.bars = o;
    o += (size_t)L.nbar * 8 + 16; // + the writer's count of records copied to global memory (u32) and the CTA's
                                  // current work item (int)
    o = (o + 127) & ~(size_t)127;
    L.rings = o;
    o += (size_t)L.nslot * rec_u16(dp) * 2;
    L.inring = o;
    o += (size_t)KI * rec_u16(dp) * 2;
    o = (o + 127) & ~(size_t)127;
    L.cring = o;
    o += (size_t)R * 2 * FB * dp * 2;
    L.total = o;
    return L;
}
// the layout of a launch of band height R (its cost copies of batch_px(dp, R) pixels)
__host__ __device__ inline SgmSmem sgm_smem(int R, int dp) { return sgm_smem_fb(R, dp, batch_px(dp, R)); }

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr uint32_t INF2 = 0x7FFF7FFFu;

// ---------------------------------------------------------------- PTX helpers
using namespace ptx;
__device__ __forceinline__ void st_release_cta_shared(uint32_t a, unsigned v) {
    asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_cta_shared(uint32_t a) {
    unsigned v;
    asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
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

// NP consecutive 32-bit words to global memory with the streaming hint (written once, read by a later kernel)
template <int NP>
__device__ __forceinline__ void stg_stream(uint16_t *p, const uint32_t (&v)[NP]) {
    if constexpr (NP % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 4; k++)
            __stcs(reinterpret_cast<uint4 *>(p) + k, make_uint4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]));
    } else if constexpr (NP % 2 == 0) {
#pragma unroll
        for (int k = 0; k < NP / 2; k++) __stcs(reinterpret_cast<uint2 *>(p) + k, make_uint2(v[2 * k], v[2 * k + 1]));
    } else {
#pragma unroll
        for (int k = 0; k < NP; k++) __stcs(reinterpret_cast<unsigned *>(p) + k, v[k]);
    }
}

// ---------------------------------------------------------------- packed path update
__device__ __forceinline__ uint32_t perm_hi_lo(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
// the smaller half of v in both halves: a warp minimum of such pairs is again a pair (m, m)
__device__ __forceinline__ uint32_t hmin2(uint32_t v) { return __vminu2(v, __byte_perm(v, 0, 0x1032)); }

// remaining-lines update of one path (sgm.cpp:278-383) for this lane's DPL = 2*NP disparities:
//   L(d) = C(d) + min(Lp(d), Lp(d-1)+7, Lp(d+1)+7, minLp+100) - minLp; returns the lane's minimum
// Per pair of disparities: one byte permute for the neighbours, min(Lp(d-1), Lp(d+1)) and min(Lp(d), minLp+100)
// as packed minima, the +7 and the final minimum as one add-then-minimum, C + m - minLp as one 3-input add;
// the lane minimum takes a 3-input packed minimum per two pairs. Every packed operation here is a single
// instruction on sm_100+ (the add-then-minimum and 3-input minimum are DPX instructions).
template <int NP>
__device__ __forceinline__ uint32_t path_step(const uint32_t (&P)[NP], uint32_t minLp, const uint32_t (&C)[NP],
                                              uint32_t (&Ln)[NP], int lane) {
    uint32_t left = __shfl_up_sync(FULL, P[NP - 1], 1);
    uint32_t right = __shfl_down_sync(FULL, P[0], 1);
    if (lane == 0) left = INF2;
    if (lane == 31) right = INF2;
    const uint32_t m2 = minLp; // (minLp, minLp)
    const uint32_t p2 = minLp + 0x00640064u;
    uint32_t xprev = perm_hi_lo(left, P[0]); // (Lp[d-1], Lp[d]) of the first pair
    uint32_t mn = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < NP; k++) {
        const uint32_t x = perm_hi_lo(P[k], (k + 1 < NP) ? P[k + 1] : right); // (Lp[d+1], Lp[d+2])
        const uint32_t m = __viaddmin_u16x2(__vminu2(xprev, x), 0x00070007u, __vminu2(P[k], p2));
        const uint32_t v = C[k] + m - m2;
        Ln[k] = v;
        if (k & 1)
            mn = __vimin3_u16x2(mn, Ln[k - 1], v);
        else if (k + 1 == NP)
            mn = __vminu2(mn, v);
        xprev = x;
    }
    return hmin2(mn);
}

// ---------------------------------------------------------------- final winner-take-all of one pixel
// The lowest d <= min(j, D-1) of S0 + S1 at padded column j (postprocess.cpp:74-185), one warp per pixel, this
// lane holding d = d0 .. d0 + 2 NP - 1: keys (sum << 16) | d; halves with d >= D or d > j are forced to sum 0xFFFF
// (real sums are smaller, and both halves of a pair are real or both infinite since dc % 8 == 0). Pixels with
// j >= dp-1 in a volume whose stride holds only real disparities (D = dp) need neither test (warp-uniform).
template <int NP>
__device__ __forceinline__ uint32_t wta_pixel(const uint32_t (&s0)[NP], const uint32_t (&s1)[NP], int d0, int j, int D,
                                              int dp) {
    uint32_t best = 0xFFFFFFFFu;
    if (j >= dp - 1 && D == dp) {
#pragma unroll
        for (int k = 0; k < NP; k++) {
            const int d = d0 + 2 * k;
            const uint32_t sv = s0[k] + s1[k];
            best = min(best, min(__byte_perm(sv, (uint32_t)d, 0x1054), __byte_perm(sv, (uint32_t)(d + 1), 0x3254)));
        }
    } else {
#pragma unroll
        for (int k = 0; k < NP; k++) {
            const int d = d0 + 2 * k;
            uint32_t sv = s0[k] + s1[k];
            if (d >= D || d > j) sv |= 0x0000FFFFu;
            if (d + 1 >= D || d + 1 > j) sv |= 0xFFFF0000u;
            best = min(best, min(__byte_perm(sv, (uint32_t)d, 0x1054), __byte_perm(sv, (uint32_t)(d + 1), 0x3254)));
        }
    }
    return __reduce_min_sync(FULL, best) & 0xFFFFu;
}

// ---------------------------------------------------------------- the kernel
// FB: pixels per cost copy, batch_px(32 * DPL, a.R)
template <int DPL, int FB>
__global__ void __launch_bounds__((rows_cap_fb(32 * DPL, FB) + kHelpers) * 32, 1) sgm_kernel(const SgmLaunch a) {
    constexpr int NP = DPL / 2;
    constexpr int KI = 2 * FB;             // incoming-ring slots
    constexpr int HB = hand_px(32 * DPL);  // pixels per full hand-off batch
    constexpr int NIB = 2 * FB / HB;       // in_batches(32 * DPL, a.R)
    extern __shared__ __align__(128) unsigned char smem[];
    const int R = a.R, dp = a.dp;
    int W = 0, H = 0; // geometry of the current work item's rig
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    const int d0 = lane * DPL;
    const int rec = rec_u16(dp);
    const SgmSmem L = sgm_smem_fb(R, dp, FB);
    const uint32_t bars = sptr(smem + L.bars);
    const uint32_t relcnt = bars + 8u * (uint32_t)L.nbar; // records of this band copied to global memory
    // ring of row w: kKP slots (kKS for the last row); slot k's full barrier at bars + 16k, empty at +8
    auto lgslots = [&](int w) { return w == R - 1 ? 3 : 2; };
    const uint32_t in_base = bars + 16u * (uint32_t)L.nslot;
    auto infull = [&](int b) { return in_base + 8u * (uint32_t)(b & (NIB - 1)); };              // batch b
    auto inempty = [&](int x) { return in_base + 8u * (uint32_t)(NIB + (x & (KI - 1))); };      // pixel x's slot
    const uint32_t c_base = in_base + 8u * (uint32_t)(NIB + KI);
    auto cfull = [&](int w, int g) { return c_base + 8u * (uint32_t)(w * 2 + (g & 1)); };
    uint16_t *rings = reinterpret_cast<uint16_t *>(smem + L.rings);
    uint16_t *inring = reinterpret_cast<uint16_t *>(smem + L.inring);
    uint16_t *cring = reinterpret_cast<uint16_t *>(smem + L.cring);

    uint32_t padm[NP]; // halves holding disparities >= dc of the current rig are infinite
    int pass = 0;      // pass of the current work item: 0 top-down left-to-right, 1 mirrored
    // cost batch b of FB pixels (q = FB*b ...) covers min(FB, W - FB*b) pixels; in memory (columns j) they
    // are contiguous, ascending in pass 0 and descending in pass 1. first column (lowest j) and pixel count:
    auto bj0 = [&](int b) { return pass ? max(0, W - FB * (b + 1)) : FB * b; };
    auto bn = [&](int b) { return min(FB, W - FB * b); };
    // Hand-off batches of the records of the band above: pixels [0,2) [2,4) then doubling up to HB, then HB at a
    // time (HB = 2: starts 0 2 4 6 ...; HB = 8: 0 2 4 8 16 24 ...), so a band can begin two pixels after the band
    // above. Each batch costs the writer a shared-memory count, the releaser a device-scope release and the
    // fetcher a poll and a copy. No batch wraps around the ring.
    constexpr int NPF = HB == 8 ? 3 : (HB == 4 ? 2 : 1); // batches before the first full one (log2 HB)
    auto hstart = [&](int b) { return b < NPF ? (b == 0 ? 0 : (1 << b)) : HB * (b - NPF + 1); };
    auto hend = [&](int b) { return min(W, hstart(b + 1)); };
    auto hbatch = [&](int x) { return x < HB ? (x < 2 ? 0 : 31 - __clz(x)) : x / HB + NPF - 1; };

    // Work items are drawn from a ticket in item order, so every item a CTA waits on (the previous band of its
    // pass) was drawn earlier by a CTA that is running or done: the launch completes however many of its CTAs
    // are resident, and needs no cooperative launch -- other kernels may share the GPU with it.
    volatile int *s_item = reinterpret_cast<volatile int *>(smem + L.bars + 8u * (uint32_t)L.nbar + 8u);
    bool first_band = true;
    for (;;) {
        if (threadIdx.x == 0) *s_item = (int)atomicAdd(a.claim, 1u);
        __syncthreads();
        const int item = *s_item;
        if (item >= a.nitems) break;
        int band, wrow = -1; // a band item (pass, band) or a final-WTA item (cropped row wrow)
        SgmRig rg;
        if (a.items) {
            const uint32_t v = a.items[item];
            rg = a.rigs[v >> 24];
            band = (int)((v >> 1) & kItemIndexMask);
            pass = (int)(v & 1u);
            if (v & kItemWta) wrow = band;
        } else {
            rg = a.rig0;
            band = item >> 1;
            pass = item & 1;
            if (item >= 2 * rg.nbands) wrow = sgm_wta_row(item - 2 * rg.nbands, rg.sh);
        }
        W = rg.W;
        H = rg.H;
        if (wrow >= 0) {
            // ===================================================== final WTA of one cropped row (fused)
            // Both passes' bands holding padded row i have published their sums (a band item releases its flag
            // after the CTA barrier that ends it); every band item was drawn before any WTA item, so the wait ends.
            const int i = rg.sy0 + wrow;
            if (threadIdx.x == 0) {
                const unsigned *f0 = rg.progress + ((size_t)(i / R)) * kProgressStride + 1;
                const unsigned *f1 = rg.progress + ((size_t)rg.nbands + (H - 1 - i) / R) * kProgressStride + 1;
                const unsigned long long t0 = global_ns();
                for (unsigned n = 0; ld_acquire(f0) == 0u || ld_acquire(f1) == 0u; n++) {
                    __nanosleep(256);
                    if (n % kCheckEvery == kCheckEvery - 1 &&
                        (ld_relaxed(a.err) != kErrNone || global_ns() - t0 > 1000ull * a.wait_limit_us)) {
                        atomicCAS(a.err, kErrNone, kErrTimeout);
                        break;
                    }
                }
            }
            __syncthreads();
            constexpr int U = 4; // pixels of one warp in flight
            const int nwarps = blockDim.x >> 5;
            const size_t rowcell = (size_t)wrow * rg.sw;
            for (int x0 = wi * U; x0 < rg.sw; x0 += nwarps * U) {
                uint32_t s0[U][NP], s1[U][NP];
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int x = min(x0 + u, rg.sw - 1);
                    const uint4 *p0 = reinterpret_cast<const uint4 *>(rg.sum0 + (rowcell + x) * dp + d0);
                    const uint4 *p1 = reinterpret_cast<const uint4 *>(rg.sum1 + (rowcell + x) * dp + d0);
                    if constexpr (NP % 4 == 0) {
#pragma unroll
                        for (int k = 0; k < NP / 4; k++) {
                            const uint4 v0 = __ldcg(p0 + k), v1 = __ldcg(p1 + k);
                            s0[u][4 * k] = v0.x; s0[u][4 * k + 1] = v0.y; s0[u][4 * k + 2] = v0.z; s0[u][4 * k + 3] = v0.w;
                            s1[u][4 * k] = v1.x; s1[u][4 * k + 1] = v1.y; s1[u][4 * k + 2] = v1.z; s1[u][4 * k + 3] = v1.w;
                        }
                    } else {
                        const unsigned *q0 = reinterpret_cast<const unsigned *>(p0), *q1 = reinterpret_cast<const unsigned *>(p1);
#pragma unroll
                        for (int k = 0; k < NP; k++) {
                            s0[u][k] = __ldcg(q0 + k);
                            s1[u][k] = __ldcg(q1 + k);
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < U; u++) {
                    const int x = x0 + u;
                    if (x >= rg.sw) break; // warp-uniform
                    const uint32_t dv = wta_pixel<NP>(s0[u], s1[u], d0, rg.sx0 + x, rg.D, dp);
                    if (lane == 0) rg.out[rowcell + x] = (uint16_t)min(dv * 255u, 0xFFFFu);
                }
            }
            __syncthreads();
            continue;
        }
#pragma unroll
        for (int k = 0; k < NP; k++)
            padm[k] = ((d0 + 2 * k < rg.D) ? 0u : 0x0000FFFFu) | ((d0 + 2 * k + 1 < rg.D) ? 0u : 0xFFFF0000u);
        const int nhb = hbatch(W - 1) + 1;
        const int nbat = (W + FB - 1) / FB;
        const uint16_t *cost = rg.cost;
        uint16_t *sum = pass ? rg.sum1 : rg.sum0;
        // hand-off rows of this pass: band b writes row b & 1, band b+1 reads it (see sgm_bnd_bytes)
        uint16_t *bnd = rg.bnd + (size_t)pass * kBndRows * W * rec;
        unsigned *progress = rg.progress + (size_t)pass * rg.nbands * kProgressStride;
        const int row0 = band * R;
        const int rows = min(R, H - row0);
        const bool publish = rows == R && band + 1 < rg.nbands;
        if (threadIdx.x == 0) {
            if (!first_band)
                for (int k = 0; k < L.nbar; k++) mbar_inval(bars + 8u * k);
            st_release_cta_shared(relcnt, 0u);
            // ring slots: producer = the row's warp, consumer = the next row's warp or, for the last row, the
            // writer (32 arrivals each)
            for (int k = 0; k < L.nslot; k++) {
                mbar_init(bars + 16u * k, 32);
                mbar_init(bars + 16u * k + 8u, 32);
            }
            for (int wr = 0; wr < R; wr++)
                for (int g = 0; g < 2; g++) mbar_init(cfull(wr, g), 1); // row warp's arrive.expect_tx + bytes
            for (int b = 0; b < NIB; b++) mbar_init(infull(b), 1);  // fetcher's arrive.expect_tx + bytes
            for (int x = 0; x < KI; x++) mbar_init(inempty(x), 32); // the first row's warp
            fence_mbar_init();
        }
        first_band = false;
        __syncthreads();

        if (wi < rows) {
            // ===================================================== row warp: all four paths of row w
            // Record of pixel q in the row's ring: r3 and m3 are stored first and the full barrier of slot q
            // is arrived on at once; r1, r2, m1, m2 follow in the same pixel and are covered by the next
            // arrival (slot q+1; after the last pixel an arrival on the slot of a virtual pixel W). The row
            // below needs r3 of column q+1 but r2 and r1 only of columns q and q-1, so it trails this row by
            // one pixel plus the r3 update rather than by a whole pixel update. At its pixel p it reads r3 of
            // column p+1 and r2, r1 of column p (r1 is kept in registers for pixel p+1) and releases column p.
            const int w = wi;
            const int r = row0 + w;
            const int i = pass ? (H - 1 - r) : r;
            const bool first_line = (r == 0);
            const bool has_cons = (w + 1 < rows) || (w == R - 1 && publish);
            const bool from_in = (w == 0); // the row above is the last row of the band above
            const int lgs = lgslots(w), ns = 1 << lgs;
            uint16_t *const oring = rings + (size_t)w * kKP * rec;
            const uint32_t obar = bars + 16u * (uint32_t)(w * kKP);
            const uint16_t *const aring = from_in ? inring : rings + (size_t)(w - 1) * kKP * rec;
            const uint32_t abar = bars + 16u * (uint32_t)((w - 1) * kKP); // rows above the last: kKP slots
            const int amask = from_in ? KI - 1 : kKP - 1;
            uint16_t *myc = cring + (size_t)w * 2 * FB * dp;
            const size_t rowbase = (size_t)i * W;
            auto prefetch = [&](int b) {
                if (lane == 0 && b < nbat) {
                    const uint32_t bytes = (uint32_t)(bn(b) * dp * 2);
                    mbar_expect_tx(cfull(w, b), bytes);
                    bulk_g2s(sptr(myc + (size_t)(b & 1) * FB * dp), cost + (rowbase + bj0(b)) * dp, bytes, cfull(w, b));
                }
            };
            // wait until column x of the row above is published up to its r3 (ring: r1 and r2 of x-1 too;
            // incoming records are whole). Called for x = 1, 2, ..., W: the incoming ring is waited on at the
            // first column of each batch and at x = 1, the first call (batch 0 holds columns 0 and 1).
            auto wait_above = [&](int x) {
                if (from_in) {
                    const int hb = hbatch(x);
                    if (x < W && (x == hstart(hb) || x == 1)) mbar_wait(infull(hb), (hb / NIB) & 1, a);
                } else {
                    mbar_wait(abar + 16u * (uint32_t)(x & (kKP - 1)), (uint32_t)(x >> 2) & 1u, a);
                }
            };
            auto release_above = [&](int x) {
                mbar_arrive(from_in ? inempty(x) : abar + 16u * (uint32_t)(x & (kKP - 1)) + 8u);
            };
            prefetch(0);
            // r0 restarts every row from Lp = 0, minLp = 0 (sgm.cpp:215-216)
            uint32_t r0[NP];
            uint32_t r0min = 0;
#pragma unroll
            for (int k = 0; k < NP; k++) r0[k] = INF2 & padm[k];
            // r1 of column q-1 of the row above (column -1: outside the image, infinite with minimum 0)
            uint32_t h1[NP];
            uint32_t hm1 = 0;
#pragma unroll
            for (int k = 0; k < NP; k++) h1[k] = INF2;
            // the pass sum is stored for pixels q in [qlo, qhi) of this row, those inside the stored window
            // (columns sx0 .. sx0+sw-1; pass 1 meets them from the right), at consecutive cells of the volume
            int sx0 = 0, sy0 = 0, sw = W, sh = H;
            if (rg.sw) {
                sx0 = rg.sx0;
                sy0 = rg.sy0;
                sw = rg.sw;
                sh = rg.sh;
            }
            const bool row_kept = i >= sy0 && i < sy0 + sh;
            const int qlo = row_kept ? (pass ? W - sx0 - sw : sx0) : 0, qhi = row_kept ? qlo + sw : 0;
            uint16_t *sp = row_kept ? sum + ((size_t)(i - sy0) * sw + (pass ? sw - 1 : 0)) * dp + d0 : sum;
            const ptrdiff_t sstep = pass ? -(ptrdiff_t)dp : (ptrdiff_t)dp;
            const uint16_t *cg = myc;
            int cn = 0;
            // unrolled by two: the second pixel takes its predecessor's states without register copies
            // (4.08 against 4.25 ms on 1920x1080/256; by four the loop outgrows the instruction cache, 4.40 ms)
#pragma unroll 2
            for (int q = 0; q < W; q++) {
                const int t = q % FB;
                if (t == 0) {
                    // group q/FB + 1 reuses the slots of group q/FB - 1, which this warp has finished
                    prefetch(q / FB + 1);
                    mbar_wait(cfull(w, q / FB), (q / FB / 2) & 1, a);
                    cg = myc + (size_t)((q / FB) & 1) * FB * dp;
                    cn = bn(q / FB);
                }
                uint32_t c[NP];
                ldw<NP>(cg + (size_t)(pass ? cn - 1 - t : t) * dp + d0, c);
                uint16_t *dst = oring + (size_t)(q & (ns - 1)) * rec;
                const uint32_t ofull = obar + 16u * (uint32_t)(q & (ns - 1));
                uint32_t n1[NP], n2[NP], n3[NP], g[NP];
                uint32_t m1, m2, m3;
                if (first_line) {
                    // First line (sgm.cpp:103-207): C' = (C == 255 ? 0 : C); r0 starts as C' and then runs the
                    // recurrence in int32 truncated to 8 bits (saturate_cast<uint16>(uint8), types.h:28);
                    // the sum receives r0 alone. r1..r3 take C' with minimum min(C') (sgm.cpp:112-114,
                    // :149-151, :192-194) and only feed the row below.
                    uint32_t cmin = 0xFFFFFFFFu;
#pragma unroll
                    for (int k = 0; k < NP; k++) {
                        n3[k] = c[k] & ~__vcmpeq2(c[k], 0x00FF00FFu);
                        cmin = __vminu2(cmin, n3[k]);
                    }
                    m3 = __reduce_min_sync(FULL, hmin2(cmin));
                    if (has_cons) {
                        stw<NP>(dst + 2 * dp + d0, n3);
                        if (lane == 0) *reinterpret_cast<uint32_t *>(dst + 3 * dp + 4) = m3;
                        mbar_arrive(ofull);
                    }
                    uint32_t mnv = 0xFFFFFFFFu;
                    if (q == 0) {
#pragma unroll
                        for (int k = 0; k < NP; k++) g[k] = n3[k];
                        mnv = cmin;
                    } else {
                        uint32_t tmp[NP];
                        path_step<NP>(r0, r0min, n3, tmp, lane);
#pragma unroll
                        for (int k = 0; k < NP; k++) {
                            g[k] = (tmp[k] & 0x00FF00FFu & ~padm[k]) | (INF2 & padm[k]);
                            mnv = __vminu2(mnv, g[k]);
                        }
                    }
#pragma unroll
                    for (int k = 0; k < NP; k++) {
                        r0[k] = g[k];
                        n1[k] = n2[k] = n3[k];
                    }
                    r0min = __reduce_min_sync(FULL, hmin2(mnv));
                    m1 = m2 = m3;
                } else {
                    // r3 reads column q+1, r2 column q, r1 column q-1 of the row above (outside the image:
                    // infinite states with minimum 0)
                    wait_above(q + 1);
                    uint32_t a2[NP], a3[NP];
                    uint32_t am2, am3 = 0;
                    if (q + 1 < W) {
                        const uint16_t *s3 = aring + (size_t)((q + 1) & amask) * rec;
                        ldw<NP>(s3 + 2 * dp + d0, a3);
                        am3 = *reinterpret_cast<const uint32_t *>(s3 + 3 * dp + 4);
                    } else {
#pragma unroll
                        for (int k = 0; k < NP; k++) a3[k] = INF2;
                    }
                    uint32_t b1[NP]; // r1 of column q, for pixel q+1
                    uint32_t bm1;
                    {
                        const uint16_t *s2 = aring + (size_t)(q & amask) * rec;
                        ldw<NP>(s2 + d0, b1);
                        ldw<NP>(s2 + dp + d0, a2);
                        const uint2 mm = *reinterpret_cast<const uint2 *>(s2 + 3 * dp);
                        bm1 = mm.x;
                        am2 = mm.y;
                        release_above(q);
                    }
                    // r3 first: the row below waits for it
                    m3 = __reduce_min_sync(FULL, path_step<NP>(a3, am3, c, n3, lane));
                    if (has_cons) {
                        stw<NP>(dst + 2 * dp + d0, n3);
                        if (lane == 0) *reinterpret_cast<uint32_t *>(dst + 3 * dp + 4) = m3;
                        mbar_arrive(ofull);
                    }
                    uint32_t n0[NP];
                    const uint32_t mn0 = path_step<NP>(r0, r0min, c, n0, lane);
                    const uint32_t mn1 = path_step<NP>(h1, hm1, c, n1, lane);
                    const uint32_t mn2 = path_step<NP>(a2, am2, c, n2, lane);
                    r0min = __reduce_min_sync(FULL, mn0);
                    m1 = __reduce_min_sync(FULL, mn1);
                    m2 = __reduce_min_sync(FULL, mn2);
#pragma unroll
                    for (int k = 0; k < NP; k++) {
                        r0[k] = n0[k];
                        g[k] = n0[k] + n1[k] + n2[k] + n3[k];
                        h1[k] = b1[k];
                    }
                    hm1 = bm1;
                }
                // the pass's sum: first line r0 alone (sgm.cpp:132, :187), else r0+r1+r2+r3 (:386-391); u16
                // arithmetic never saturates or wraps for real disparities
                if ((unsigned)(q - qlo) < (unsigned)(qhi - qlo)) {
                    stg_stream<NP>(sp, g);
                    sp += sstep;
                }
                if (has_cons) {
                    stw<NP>(dst + d0, n1);
                    stw<NP>(dst + dp + d0, n2);
                    if (lane == 0) *reinterpret_cast<uint2 *>(dst + 3 * dp) = make_uint2(m1, m2);
                    // the slots of pixels q+1 and q+2 last held pixels q+1-ns and q+2-ns; at even q one wait for the
                    // later release covers both (the row below releases in pixel order)
                    const int y = q + 2 - ns;
                    if (!(q & 1) && y >= 0)
                        mbar_wait(obar + 16u * (uint32_t)((q + 2) & (ns - 1)) + 8u, (uint32_t)(y >> lgs) & 1u, a);
                }
            }
            // virtual pixel W: publishes r1 and r2 of the last pixel
            if (has_cons) mbar_arrive(obar + 16u * (uint32_t)(W & (ns - 1)));
            // every copy this warp issued has been waited for; after a timeout a wait may have returned
            // early, so make sure none is still in flight before the barriers are reused
            if (lane == 0)
                for (int b = max(0, nbat - 2); b < nbat; b++) mbar_drain(cfull(w, b), (b / 2) & 1, kDrainLimitUs);
        } else if (wi == R && band > 0) {
            // ===================================================== fetcher: records of the band above -> inring
            if (lane == 0) {
                const uint16_t *src = bnd + (size_t)((band - 1) & (kBndRows - 1)) * W * rec;
                const unsigned *prog = progress + (size_t)(band - 1) * kProgressStride;
                unsigned seen = 0;
                for (int b = 0; b < nhb; b++) {
                    const int hs = hstart(b), he = hend(b), nb = he - hs;
                    // before reusing barrier b % NIB the reader must be past batch b-NIB, and the ring slots of
                    // pixels hs..he-1 must be free (they last held pixels hs-KI..he-1-KI); the reader releases
                    // in pixel order, so waiting for the later of the two last pixels covers both
                    const int y = max(b >= NIB ? hend(b - NIB) - 1 : -1, he - 1 - KI);
                    if (y >= 0) mbar_wait(inempty(y), (y / KI) & 1, a);
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
                    bulk_g2s(sptr(inring + (size_t)(hs % KI) * rec), src + (size_t)hs * rec, bytes, infull(b));
                }
                for (int b = max(0, nhb - NIB); b < nhb; b++) mbar_drain(infull(b), (b / NIB) & 1, kDrainLimitUs);
            }
        } else if (wi == R + 1 && publish) {
            // ===================================================== writer: band's last row -> global memory
            // record x is complete once the last row has arrived on the slot of x+1 (x = W-1: virtual pixel W).
            // At the end of every hand-off batch the count of copied records goes to the releaser through
            // shared memory; the writer itself never waits on a device-wide fence.
            uint16_t *dst = bnd + (size_t)(band & (kBndRows - 1)) * W * rec;
            const uint16_t *lring = rings + (size_t)(R - 1) * kKP * rec;
            const uint32_t lbar = bars + 16u * (uint32_t)((R - 1) * kKP);
            const int nch = rec / 8; // 16-byte chunks per record
            for (int x = 0; x < W; x++) {
                mbar_wait(lbar + 16u * (uint32_t)((x + 1) & (kKS - 1)), (uint32_t)((x + 1) >> 3) & 1u, a);
                const uint4 *s4 = reinterpret_cast<const uint4 *>(lring + (size_t)(x & (kKS - 1)) * rec);
                uint4 *g4 = reinterpret_cast<uint4 *>(dst + (size_t)x * rec);
                for (int k = lane; k < nch; k += 32) g4[k] = s4[k];
                mbar_arrive(lbar + 16u * (uint32_t)(x & (kKS - 1)) + 8u);
                if (x + 1 == hend(hbatch(x))) {
                    // the other lanes' stores are ordered before lane 0's release through the warp barrier
                    __syncwarp();
                    if (lane == 0) st_release_cta_shared(relcnt, (unsigned)(x + 1));
                }
            }
        } else if (wi == R + 2 && publish && lane == 0) {
            // ===================================================== releaser: copied records -> progress counter
            // A device-scope release of the latest count (cumulative: it covers the writer's stores, which this
            // thread acquired through the shared counter); batches that completed while a release was in flight
            // are published together by the next one.
            unsigned last = 0;
            const unsigned long long t0 = global_ns();
            for (unsigned n = 0; last < (unsigned)W; n++) {
                const unsigned v = ld_acquire_cta_shared(relcnt);
                if (v > last) {
                    st_release(progress + (size_t)band * kProgressStride, v);
                    last = v;
                    continue;
                }
                __nanosleep(64);
                if (n % kCheckEvery == kCheckEvery - 1 &&
                    (ld_relaxed(a.err) != kErrNone || global_ns() - t0 > 1000ull * a.wait_limit_us)) {
                    atomicCAS(a.err, kErrNone, kErrTimeout);
                    break;
                }
            }
        }
        __syncthreads();
        // a band item's sums are complete: release its flag for the fused WTA items of its rows
        if (rg.out && threadIdx.x == 0) {
            __threadfence();
            st_release(progress + (size_t)band * kProgressStride + 1, 1u);
        }
    }
}

// Sum of the two passes' sums and the final WTALeft (hpp:283, postprocess.cpp:74-185): the lowest
// d <= min(j, dc-1) of S0 + S1 (pass 1 adds its sum to pass 0's, saturating at sgm.cpp:390 -- real sums
// stay below 2 * 4 * 1121, so nothing saturates), then crop and *255 (hpp:111-118). One warp per pixel, lanes
// over d; memory-bound. Without a padded map to fill (disp null) only the cropped pixels are computed, which
// reads the sum volumes over w*h pixels instead of Wp*Hp.
template <int DPL>
__global__ void __launch_bounds__(256) sgm_wta_kernel(const uint16_t *__restrict__ s0v, const uint16_t *__restrict__ s1v,
                                                      Geom g, uint16_t *__restrict__ out, uint16_t *__restrict__ disp,
                                                      bool cropped) {
    constexpr int NP = DPL / 2;
    const int lane = threadIdx.x & 31;
    const size_t t = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    int i, j;
    if (disp) {
        if (t >= g.plane) return;
        i = (int)(t / g.Wp);
        j = (int)(t % g.Wp);
    } else {
        if (t >= (size_t)g.w * g.h) return;
        i = (int)(t / g.w) + g.dc;
        j = (int)(t % g.w) + g.dc;
    }
    const size_t pix = (size_t)i * g.Wp + j;
    const size_t cell = cropped ? t : pix; // stored sums: the original image only (row-major, w per row) or the plane
    const int d0 = lane * DPL, D = g.dc;
    uint32_t s0[NP], s1[NP];
    ldw<NP>(s0v + cell * g.dp + d0, s0);
    ldw<NP>(s1v + cell * g.dp + d0, s1);
    const uint32_t dv = wta_pixel<NP>(s0, s1, d0, j, D, g.dp);
    if (lane == 0) {
        if (disp) disp[pix] = (uint16_t)dv;
        const int oi = i - g.dc, oj = j - g.dc;
        if (out && oi >= 0 && oi < g.h && oj >= 0 && oj < g.w) out[(size_t)oi * g.w + oj] = (uint16_t)min(dv * 255u, 0xFFFFu);
    }
}

// WTARight_SSE with uniqueness 1 (postprocess.cpp:187-315) on S0 + S1, for the two-view doStereo (hpp:139):
// R(i, b) = the lowest k <= min(dc-1, W-1-b) minimising S(i, b+k, k). One warp per pixel, lanes over k; the cells
// lie on a diagonal of the volume (stride dp + 1), which only this path reads.
template <int DPL>
__global__ void __launch_bounds__(256) sgm_wta_right_kernel(const uint16_t *__restrict__ s0v,
                                                            const uint16_t *__restrict__ s1v, Geom g,
                                                            uint16_t *__restrict__ disp) {
    const int lane = threadIdx.x & 31;
    const size_t pix = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (pix >= g.plane) return;
    const int b = (int)(pix % g.Wp);
    const int end = min(g.dc - 1, g.Wp - 1 - b);
    uint32_t best = 0xFFFFFFFFu;
#pragma unroll
    for (int t = 0; t < DPL; t++) {
        const int k = lane * DPL + t;
        if (k <= end) {
            const size_t cell = (pix + k) * g.dp + k;
            best = min(best, ((uint32_t)(s0v[cell] + s1v[cell]) << 16) | (uint32_t)k);
        }
    }
    best = __reduce_min_sync(FULL, best);
    if (lane == 0) disp[pix] = (uint16_t)(best & 0xFFFFu);
}

// the instantiation for dpl disparities per lane and bands of R rows (R = 0: the one with the widest cost groups)
const void *kernel_for(int dpl, int R) {
    switch (dpl) {
    case 2: return (const void *)sgm_kernel<2, batch_px(64, 1)>;
    case 4: return (const void *)sgm_kernel<4, batch_px(128, 1)>;
    case 6: return (const void *)sgm_kernel<6, batch_px(192, 1)>;
    case 8: return (const void *)sgm_kernel<8, batch_px(256, 1)>;
    case 12: return (const void *)sgm_kernel<12, batch_px(384, 1)>;
    case 16: return batch_px(512, R) == 2 ? (const void *)sgm_kernel<16, 2> : (const void *)sgm_kernel<16, 4>;
    default: return nullptr;
    }
}

} // namespace

void init_sgm_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    for (int dpl : kDplChoices)
        for (int R : {1, rows_cap(32 * dpl)})
            cudaFuncSetAttribute(kernel_for(dpl, R), cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    cudaGetLastError();
    init_cost_kernels();
}

// largest band height whose shared-memory layout fits this device
int sgm_rows_max(int dp, int device) {
    int optin = 227 * 1024;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    cudaGetLastError();
    int rmax = rows_cap(dp);
    while (rmax > 1 && sgm_smem(rmax, dp).total > (size_t)optin) rmax--;
    return rmax;
}

// largest band height on a GB300 (227 KB of shared memory per CTA), without a device query
int sgm_rows_gb300(int dp) {
    int rmax = rows_cap(dp);
    while (rmax > 1 && sgm_smem(rmax, dp).total > 227 * 1024) rmax--;
    return rmax;
}

namespace {
// Rows per band. The plan simulates the persistent schedule: work item k (band k >> 1 of pass k & 1) runs on
// CTA k mod (resident CTAs) after that CTA's previous item, and no earlier than one band lag after the
// previous band of its pass; an item takes W pixel periods. A row warp's pixel period grows with the row
// warps that share its scheduler (four schedulers per SM; warp w runs on scheduler w mod 4, so the busiest one
// carries ceil(rows per SM / 4)) above a latency floor, and the band lag is about 1.33 periods per row plus the
// hand-off (a 2-pixel batch of records, its release, poll and copy: about 7 periods), so in units of one row's
// issue time: period T = 20 + 4 ceil(rows per SM / 4), band lag = (1.33 R + 7) T. The band height with the
// earliest simulated finish wins; ties go to the taller band (fewer hand-offs). per_sm(R): CTAs of band height
// R per SM.
template <class F>
SgmPlan plan_rows(const Geom &g, int sms, int lo, int hi, F per_sm) {
    SgmPlan p{};
    double best = 0;
    std::vector<double> free, start;
    for (int R = hi; R >= lo; R--) {
        const int k = per_sm(R);
        if (k < 1) continue;
        const int nb = (g.Hp + R - 1) / R;
        const int items = 2 * nb;
        const int conc = std::min(items, k * sms);
        const int rows_sm = R * ((conc + sms - 1) / sms);
        const double T = 20.0 + 4.0 * ((rows_sm + 3) / 4);
        const double lag = (1.33 * R + 7.0) * T, sweep = (double)g.Wp * T;
        free.assign(conc, 0.0);
        start.assign(items, 0.0);
        double end = 0;
        for (int it = 0; it < items; it++) {
            double s0 = free[it % conc];
            if (it >= 2) s0 = std::max(s0, start[it - 2] + lag);
            start[it] = s0;
            free[it % conc] = s0 + sweep;
            end = std::max(end, s0 + sweep);
        }
        if (p.R == 0 || end < best) {
            best = end;
            p.R = R;
            p.nbands = nb;
            p.ngroups = items;
            p.nclusters = conc; // persistent CTAs (the grid)
        }
    }
    p.cs = p.R ? 1 : 0;
    return p;
}
} // namespace

// Launch plan on `device`; force_R fixes the band height (tuning). ngroups counts the work items of one
// launch (two passes x nbands), each with a progress counter and a hand-off record row.
SgmPlan sgm_plan(const Geom &g, int device, int force_R, int /*force_cs: bands are never clustered*/) {
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaGetLastError();
    if (!kernel_for(g.dpl, 1)) return SgmPlan{};
    const int rmax = sgm_rows_max(g.dp, device);
    // on a 152-SM GB300, the band height the autotuner measured fastest for this geometry's class
    if (!force_R && sms == 152)
        for (const TunedRows &t : kTunedRows)
            if (t.dp == g.dp && g.Hp >= t.hp_lo && g.Hp < t.hp_hi && t.rows >= 1 && t.rows <= rmax) {
                force_R = t.rows;
                break;
            }
    const int lo = force_R ? std::max(1, std::min(rmax, force_R)) : 1;
    return plan_rows(g, sms, lo, force_R ? lo : rmax, [&](int R) {
        int k = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, kernel_for(g.dpl, R), (R + kHelpers) * 32,
                                                          sgm_smem(R, g.dp).total) != cudaSuccess) {
            cudaGetLastError();
            k = 0;
        }
        return k;
    });
}

// The same plan for a 152-SM GB300 without a device query (227 KB of shared memory per CTA, 228 KB and 64
// warps per SM): used for memory estimates.
SgmPlan sgm_plan_gb300(const Geom &g) {
    if (!kernel_for(g.dpl, 1)) return SgmPlan{};
    return plan_rows(g, 152, 1, sgm_rows_gb300(g.dp), [&](int R) {
        return (int)std::min<size_t>(228 * 1024 / (sgm_smem(R, g.dp).total + 1024), 64 / (R + kHelpers));
    });
}

// Hand-off records: kBndRows rows of Wp records per pass, band b writing row b % kBndRows. Two rows suffice: band
// b+2 writes record x only after its last row reached pixel x, which trails its first row by R-1 pixels, which
// trails band b+1's last row, which trails band b+1's first row by R-1 more; so band b+1's first row has passed
// pixel x + 2R - 1 by then, and it processes a pixel only after its fetcher's copy of that record from band b's row
// has landed in shared memory. (An expired wait breaks the chain, but then the result is reported as a timeout.)
size_t sgm_bnd_bytes(const Geom &g, const SgmPlan &) {
    return (size_t)2 * kBndRows * g.Wp * rec_u16(g.dp) * sizeof(uint16_t);
}

cudaError_t launch_sgm(const Geom &g, const SgmPlan &p, SgmRig rig, unsigned *err, cudaStream_t st,
                       unsigned wait_limit_us) {
    if (p.R < 1) return cudaErrorInvalidConfiguration;
    const void *fn = kernel_for(g.dpl, p.R);
    if (!fn) return cudaErrorInvalidValue;
    rig.W = g.Wp;
    rig.H = g.Hp;
    rig.D = g.dc;
    rig.nbands = p.nbands;
    SgmLaunch a{};
    a.rig0 = rig;
    a.rigs = nullptr;
    a.items = nullptr;
    if (rig.out && rig.sw == 0) return cudaErrorInvalidValue; // the fused WTA reads sums of the original image
    a.nitems = p.ngroups + (rig.out ? rig.sh : 0);
    a.R = p.R;
    a.dp = g.dp;
    a.claim = rig.progress + (size_t)p.ngroups * kProgressStride;
    a.err = err;
    a.wait_limit_us = wait_limit_us;
    cudaError_t e = cudaMemsetAsync(rig.progress, 0, sgm_progress_bytes(p.ngroups), st);
    if (e != cudaSuccess) return e;
    void *args[] = {(void *)&a};
    // each work item depends only on items drawn before it (the previous band of its pass), so a plain launch
    // of any grid size completes
    return cudaLaunchKernel(fn, dim3(p.nclusters), dim3((p.R + kHelpers) * 32), args, sgm_smem(p.R, g.dp).total, st);
}

void sgm_build_items(const SgmItemRig *rigs, int nrigs, int R, bool fuse, std::vector<uint32_t> &items) {
    items.clear();
    int maxb = 0;
    for (int k = 0; k < nrigs; k++) maxb = std::max(maxb, rigs[k].nbands);
    // position of band item (rig k, pass, band) in the band order: first[k][band] + pass
    std::vector<std::vector<int>> first(nrigs);
    for (int k = 0; k < nrigs; k++) first[k].assign(rigs[k].nbands, 0);
    for (int band = 0; band < maxb; band++)
        for (int k = 0; k < nrigs; k++)
            if (band < rigs[k].nbands) {
                first[k][band] = (int)items.size();
                for (int pass = 0; pass < 2; pass++) items.push_back(sgm_item_band(k, band, pass));
            }
    if (!fuse) return;
    struct W {
        int key;  // position of the later of the row's two band items
        int dist; // distance of the row from its rig's middle row (ties: nearest the middle first)
        uint32_t item;
    };
    std::vector<W> ws;
    for (int k = 0; k < nrigs; k++)
        for (int c = 0; c < rigs[k].sh; c++) {
            const int i = rigs[k].sy0 + c;
            const int e = std::max(first[k][i / R], first[k][(rigs[k].H - 1 - i) / R] + 1);
            ws.push_back({e, std::abs(2 * c + 1 - rigs[k].sh), sgm_item_wta(k, c)});
        }
    std::stable_sort(ws.begin(), ws.end(), [](const W &a, const W &b) {
        return a.key != b.key ? a.key < b.key : a.dist < b.dist;
    });
    for (const W &w : ws) items.push_back(w.item);
}

cudaError_t launch_sgm_multi(int dp, int R, const SgmRig *rigs_dev, const uint32_t *items_dev, int nitems,
                             unsigned *claim, unsigned *err, int device, cudaStream_t st, unsigned wait_limit_us) {
    const int dpl = dp / 32;
    const void *fn = kernel_for(dpl, R);
    if (!fn || R < 1 || nitems < 1) return cudaErrorInvalidValue;
    int sms = 152, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (R + kHelpers) * 32, sgm_smem(R, dp).total) !=
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
    a.claim = claim;
    a.err = err;
    a.wait_limit_us = wait_limit_us;
    void *args[] = {(void *)&a};
    return cudaLaunchKernel(fn, dim3(std::min(nitems, per_sm * sms)), dim3((R + kHelpers) * 32), args,
                            sgm_smem(R, dp).total, st);
}

cudaError_t launch_sgm_wta_right(const Geom &g, const uint16_t *s0, const uint16_t *s1, uint16_t *disp,
                                 cudaStream_t st) {
    const unsigned blocks = (unsigned)((g.plane + 7) / 8);
    switch (g.dpl) {
    case 2: sgm_wta_right_kernel<2><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    case 4: sgm_wta_right_kernel<4><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    case 6: sgm_wta_right_kernel<6><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    case 8: sgm_wta_right_kernel<8><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    case 12: sgm_wta_right_kernel<12><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    case 16: sgm_wta_right_kernel<16><<<blocks, 256, 0, st>>>(s0, s1, g, disp); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_sgm_wta(const Geom &g, const uint16_t *s0, const uint16_t *s1, uint16_t *out, uint16_t *disp,
                           cudaStream_t st, bool cropped) {
    if (cropped && disp) return cudaErrorInvalidValue; // a padded map needs the sums of the whole plane
    const unsigned blocks = (unsigned)(((disp ? g.plane : (size_t)g.w * g.h) + 7) / 8);
    switch (g.dpl) {
    case 2: sgm_wta_kernel<2><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    case 4: sgm_wta_kernel<4><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    case 6: sgm_wta_kernel<6><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    case 8: sgm_wta_kernel<8><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    case 12: sgm_wta_kernel<12><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    case 16: sgm_wta_kernel<16><<<blocks, 256, 0, st>>>(s0, s1, g, out, disp, cropped); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

} // namespace sister
