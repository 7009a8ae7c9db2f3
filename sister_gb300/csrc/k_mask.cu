// Confidence-mask kernels: per-pair WTA-left/right from census words, the reference's in-place
// (row-recursive) 3x3 median, LR check and the per-pair masks in padded original coordinates.
#include "sister_internal.h"
#include "ptx_sync.h"

namespace sister {
namespace {
using namespace ptx;

// WTALeft_SSE / WTARight_SSE with uniqueness 1 (postprocess.cpp:74-315) on a pair's Hamming volume
// (census.cpp:54-146), without materialising the volume. Both reduce to the lowest-index argmin of the
// same keys over the band 0 <= d = a - b < D of a frame row:
//   L(a) = min over b of key(a, b)   (d = a - b <= min(a, D-1))
//   R(b) = min over a of key(a, b)   (k = a - b <= min(D-1, W-1-b))
// so every cell is counted once. Keys are 16 bits, popc(Cc[a] ^ Cn[b]) << 9 | d (popcount <= 64, d < 512): the
// lowest key is the lowest cost and, among equal costs, the lowest d, which is the reference's tie rule. Two keys
// share each 32-bit word, so every packed minimum and every shuffle serves two cells.
// Rows 0..2 (all 255) and rows H-2, H-1 (never written, defined 0) have constant costs: argmin 0.
// One CTA per frame row; the centre census row is staged in shared memory, and the row's band is cut into work
// units of 64 columns x 64 diagonals spread over the CTA's warps.
// In a unit, lane l holds the adjacent columns cA = b0+2l and cB = cA+1 and walks the diagonals four per step.
// At step d it meets cells A_i = (cA+d+i, cA) and B_i = (cB+d+i, cB), i = 0..3: eight cells from the five words
// Cc[cA+d .. cA+d+4] (cA+d is even, so two 16-byte loads and one 8-byte load). R of both columns stays in a
// register. Lane l carries the partial L of the row pair (cA+d, cA+d+1). That pair's cells this step are A0, and
// A1 and B0, of lane l; A2 and B1, A3 and B2 of lane l-1; and B3 of lane l-2: lane l sends U = (min(A2, B1),
// min(A3, B2)) to lane l+1 and V = (B3, -) to lane l+2. Lanes 0 and 1 receive, wrapping around, the cells of the
// pairs that enter the warp after the step. After the step the pairs of lanes 0 and 1 (rows b0+d .. b0+d+3) have
// no later cell in this unit: they are merged into shared memory, and the partials move two lanes down, lanes 30
// and 31 taking the entering pairs. Partials still held at the end of a unit and the R of its columns are merged
// too (shared atomicMin). d0 and d1 are multiples of 4.
constexpr unsigned FULLW = 0xFFFFFFFFu;
constexpr int kWtaCols = 64, kWtaDiags = 64; // a work unit

__device__ __forceinline__ uint32_t mad_u32(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}
// (popc(xa) << 9 | d, popc(xb) << 9 | d) from the two 64-bit XOR words: four multiply-adds of the halves' popcounts
// (the halves never overlap: popcounts <= 64, d < 512), which keep the key off the integer ALU pipe
__device__ __forceinline__ uint32_t keypair(uint64_t xa, uint64_t xb, uint32_t dd) {
    const uint32_t t1 = mad_u32((uint32_t)__popc((uint32_t)(xb >> 32)), 65536u, (uint32_t)__popc((uint32_t)(xa >> 32)));
    const uint32_t t2 = mad_u32((uint32_t)__popc((uint32_t)xb), 65536u, (uint32_t)__popc((uint32_t)xa));
    return mad_u32(t1, 512u, mad_u32(t2, 512u, dd));
}

template <bool EDGE>
__device__ __forceinline__ void wta_unit(const uint64_t *cc, uint64_t wA, uint64_t wB, int b0, int lane, int W,
                                         int d0, int d1, uint32_t *lk, uint32_t *rk, uint32_t *done) {
    const int cA = b0 + 2 * lane, cB = cA + 1;
    uint32_t lacc = FULLW, racc = FULLW;
    // OR masks: a received U (V) counts for this lane's pair when lane >= 1 (2), else for an entering pair
    const uint32_t mU = lane >= 1 ? 0u : ~0u, mV = lane >= 2 ? 0u : ~0u;
    // words cA+d and cA+d+1 of the next step: the previous step loaded them (two 16-byte loads per step; without
    // EDGE the last step's second word may be the first word after the row, the key array in shared memory, never
    // used)
    uint64_t n0, n1;
    if (EDGE) {
        n0 = cc[min(cA + d0, W - 1)];
        n1 = cc[min(cA + d0 + 1, W - 1)];
    } else {
        const ulonglong2 p = *reinterpret_cast<const ulonglong2 *>(cc + cA + d0);
        n0 = p.x;
        n1 = p.y;
    }
#pragma unroll 4
    for (int d = d0; d < d1; d += 4) {
        uint64_t c[6];
        c[0] = n0;
        c[1] = n1;
        if (EDGE) {
#pragma unroll
            for (int t = 2; t < 6; t++) c[t] = cc[min(cA + d + t, W - 1)];
        } else {
            const ulonglong2 p23 = *reinterpret_cast<const ulonglong2 *>(cc + cA + d + 2);
            const ulonglong2 p45 = *reinterpret_cast<const ulonglong2 *>(cc + cA + d + 4);
            c[2] = p23.x; c[3] = p23.y; c[4] = p45.x; c[5] = p45.y;
        }
        n0 = c[4];
        n1 = c[5];
        uint32_t kab[4]; // (A_i, B_i)
#pragma unroll
        for (int i = 0; i < 4; i++) {
            kab[i] = keypair(c[i] ^ wA, c[i + 1] ^ wB, (uint32_t)(d + i) * 0x10001u);
            if (EDGE) {
                if (cA + d + i >= W) kab[i] |= 0x0000FFFFu;
                if (cB + d + i >= W) kab[i] |= 0xFFFF0000u;
            }
        }
        racc = __vimin3_u16x2(__vimin3_u16x2(racc, kab[0], kab[1]), kab[2], kab[3]);
        const uint32_t own = __vminu2(__byte_perm(kab[0], kab[1], 0x5410), kab[0] | 0x0000FFFFu); // (A0, min(A1, B0))
        const uint32_t u = __vminu2(__byte_perm(kab[2], kab[3], 0x5410), __byte_perm(kab[1], kab[2], 0x7632));
        const uint32_t v = __byte_perm(kab[3], 0xFFFFFFFFu, 0x7632); // (B3, -)
        const uint32_t ur = __shfl_sync(FULLW, u, (lane + 31) & 31);
        const uint32_t vr = __shfl_sync(FULLW, v, (lane + 30) & 31);
        lacc = __vminu2(__vimin3_u16x2(lacc, own, ur | mU), vr | mV);
        const uint32_t ent = __vminu2(ur | ~mU, vr | ~mV);
        // rows cA+d and cA+d+1 (< W: the unit's rows stay below b0 + dmax) are complete here: lanes 0 and 1 hold rows
        // b0+d .. b0+d+3, kept in the warp's buffer (word (d - d0)/2 + lane) and merged after the unit
        if (lane < 2) done[((d - d0) >> 1) + lane] = lacc;
        lacc = __shfl_sync(FULLW, lane < 2 ? ent : lacc, (lane + 2) & 31);
    }
    __syncwarp();
    if (2 * lane < d1 - d0) { // rows b0+d0 .. b0+d1-1, two per lane
        const uint32_t w = done[lane];
        atomicMin(&lk[b0 + d0 + 2 * lane], w & 0xFFFFu);
        atomicMin(&lk[b0 + d0 + 2 * lane + 1], w >> 16);
    }
    __syncwarp(); // the buffer is free for the warp's next unit
    // lane l now carries rows cA+d1 and cA+d1+1, which may have cells in other units
    if (cA + d1 < W && (lacc & 0xFFFFu) != 0xFFFFu) atomicMin(&lk[cA + d1], lacc & 0xFFFFu);
    if (cA + d1 + 1 < W && (lacc >> 16) != 0xFFFFu) atomicMin(&lk[cA + d1 + 1], lacc >> 16);
    if (cA < W) atomicMin(&rk[cA], racc & 0xFFFFu);
    if (cB < W) atomicMin(&rk[cB], racc >> 16);
}

// With rowflags, each block publishes its frame row when both maps' rows are written: rowflags[f * max(Wp, Hp) +
// i] = epoch (release), so that the frame's median can start on the first rows while later rows are computed.
// Shared memory: the centre census row (W words), the L and R key arrays (2 W u32) and 32 u32 per warp; the
// neighbour row's words are read from global memory, two per lane and work unit.
__device__ __forceinline__ void pair_wta_row(const uint64_t *__restrict__ census, const Geom &g,
                                             uint16_t *__restrict__ wta, int f, int i, unsigned *rowflags,
                                             unsigned epoch, uint64_t *srow) {
    const int H = g.frows(f), W = g.fcols(f), D = g.dc;
    uint16_t *L = wta + (size_t)(2 * f) * g.plane + (size_t)i * W;
    uint16_t *R = wta + (size_t)(2 * f + 1) * g.plane + (size_t)i * W;
    if (i < 3 || i >= H - 2) {
        for (int j = threadIdx.x; j < W; j += blockDim.x) {
            L[j] = 0;
            R[j] = 0;
        }
    } else {
        uint64_t *cc = srow;
        uint32_t *lk = reinterpret_cast<uint32_t *>(srow + W), *rk = lk + W;
        const uint64_t *gc = census + (size_t)(2 * f) * g.plane + (size_t)i * W;
        const uint64_t *gn = census + (size_t)(2 * f + 1) * g.plane + (size_t)i * W;
        for (int j = threadIdx.x; j < W; j += blockDim.x) {
            cc[j] = gc[j];
            lk[j] = FULLW;
            rk[j] = FULLW;
        }
        __syncthreads();
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        uint32_t *done = rk + W + 32 * warp; // the warp's completed rows of a unit
        const int nblk = (W + kWtaCols - 1) / kWtaCols, nch = (D + kWtaDiags - 1) / kWtaDiags;
        for (int u = warp; u < nblk * nch; u += nw) {
            const int blk = u / nch, ch = u - blk * nch;
            const int b0 = kWtaCols * blk;
            const int dmax = min(D, W - b0); // a multiple of 4 (D of 8, W of 4, b0 of 64)
            const int d0 = kWtaDiags * ch, d1 = min(d0 + kWtaDiags, dmax);
            if (d0 >= d1) continue; // warp-uniform
            // the unit's two neighbour words per lane come straight from global memory (read-only here)
            const uint64_t wA = __ldg(gn + min(b0 + 2 * lane, W - 1)), wB = __ldg(gn + min(b0 + 2 * lane + 1, W - 1));
            // the unit reads words up to cA + d1 (lane 31: b0 + 62 + d1)
            if (b0 + kWtaCols - 2 + d1 < W) wta_unit<false>(cc, wA, wB, b0, lane, W, d0, d1, lk, rk, done);
            else wta_unit<true>(cc, wA, wB, b0, lane, W, d0, d1, lk, rk, done);
        }
        __syncthreads();
        for (int j = threadIdx.x; j < W; j += blockDim.x) {
            L[j] = (uint16_t)(lk[j] & 0x1FFu);
            R[j] = (uint16_t)(rk[j] & 0x1FFu);
        }
    }
    if (rowflags) {
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            st_release(rowflags + (size_t)f * max(g.Wp, g.Hp) + i, epoch);
        }
    }
}

// shared ring length for the median sweep: a power of two >= 2W
__host__ __device__ inline int median_ring(int W) {
    int r = 1;
    while (r < 2 * W) r <<= 1;
    return r;
}

// Packed median helpers: two u16 map values per 32-bit word. Map values are disparities <= 511, so the sum
// of three fits a half and the median of three is a + b + c - min - max with no half carrying or borrowing;
// the 3-input packed minimum and maximum are single DPX instructions on sm_100+.
__device__ __forceinline__ uint32_t pmed3(uint32_t a, uint32_t b, uint32_t c) {
    return a + b + c - __vimin3_u16x2(a, b, c) - __vimax3_u16x2(a, b, c);
}
// (high half of a, low half of b): the column pair shifted by one position
__device__ __forceinline__ uint32_t shift1(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
constexpr int kMedPairsMax = 2; // packed position pairs per thread in a pass over a chunk (1 or 2, per map)

// median3x3_SSE(a, a, W, H) in place (postprocess.cpp:15-71 as called at SisterMultiviewDisparities.hpp:198
// and siblings). Over the flattened array of N = W*H: out[x] = in[x] for x < W and x >= N-W-4;
// out[W] = 0; for W < x < N-W-4, out[x] = med9(out[x-W-1], out[x-W], out[x-W+1], in[x-1], in[x], in[x+1],
// in[x+W-1], in[x+W], in[x+W+1]) where the first three were already filtered in the same sweep.
// out[x] depends only on positions <= x-W+1, so chunks of W-1 consecutive positions are independent:
// one CTA per map sweeps the chunks in order, keeping the last 2W outputs in a shared ring. The inputs
// a chunk reads (positions s-1 .. e+W) are staged in shared memory by cp.async kMedPF chunks ahead into
// kMedPF+1 buffers, so the sweep never waits on global memory and needs one CTA barrier per chunk.
// Inside a chunk the positions are taken in even-aligned pairs, two per 32-bit word: window column c of
// position x is (out[c-W], in[c], in[c+W]); each packed column word is sorted once (packed min, median, max)
// and the median of nine is med3(max of the column minima, med3 of the column medians, min of the column
// maxima), the shifted columns coming from byte permutes of neighbouring words. An odd first position s is the
// high half of the pair (s-1, s) and an odd last one e-1 the low half of (e-1, e): only that half is stored (s-1
// belongs to the previous chunk, and e depends on the chunk's first position), so every thread of a chunk runs
// the same packed code. Halves of loaded words outside the chunk's columns only feed halves that are not stored;
// they hold map values too (shared memory is zeroed first), so they cannot carry into a stored half.
// With rowflags the kernel may run while the frame's pair WTA is still writing the map: before input rows are
// read (the head, each chunk's staging, the tail) warp 0 waits until they are published with this epoch,
// and a CTA barrier passes that on. The wait is bounded: on expiry the error flag is raised and the sweep goes on.
constexpr int kMedPF = 3;
template <int kMedPairs>
__device__ __forceinline__ void median_map(const uint16_t *__restrict__ wta, const Geom &g, uint16_t *__restrict__ med,
                                           int k, const unsigned *rowflags, unsigned epoch, unsigned *err,
                                           uint16_t *msm) {
    const int f = k >> 1;
    const int H = g.frows(f), W = g.fcols(f);
    const int N = W * H; // a multiple of 16 (W and H are multiples of 4)
    const uint16_t *in = wta + (size_t)k * g.plane;
    uint16_t *out = med + (size_t)k * g.plane;
    const int rlen = median_ring(W), mask = rlen - 1;
    const int blen = 2 * W + 32; // staged input span of one chunk, rounded out to 16-byte boundaries
    uint16_t *ring = msm;        // ring[x & mask] = out[x] for the last 2W positions
    uint16_t *bufs = msm + rlen; // kMedPF + 1 staging buffers of blen
    // every shared entry starts at 0, so that the halves of packed words which hold no position of the chunk
    // (never-written entries included) are map values <= 511 like all others and no packed sum carries
    for (int o = threadIdx.x; o < (rlen + (kMedPF + 1) * blen) / 2; o += blockDim.x) reinterpret_cast<uint32_t *>(msm)[o] = 0u;
    const unsigned *flags = rowflags ? rowflags + (size_t)f * max(g.Wp, g.Hp) : nullptr;
    int ready = 0; // (warp 0) input rows known to be published
    // warp 0, until the rows holding positions up to idx are published: it reads 32 consecutive row flags per poll
    // and advances past the leading published ones. While the rows are known published the call costs a compare
    // (no division by W in the sweep: at 640x480/192 the pair WTA + median stage 0.52 -> 0.47 ms). Reading the
    // next flags ahead with relaxed loads and a fence measured slower.
    auto wait_upto = [&](int idx) {
        if (!flags || threadIdx.x >= 32 || idx < ready * W) return;
        const int lane = threadIdx.x;
        const int last = min(idx / W, H - 1);
        const unsigned long long t0 = global_ns();
        for (unsigned n = 1; ready <= last; n++) {
            const int r = ready + lane;
            const unsigned ok = __ballot_sync(0xFFFFFFFFu, r >= H || ld_acquire(flags + r) == epoch);
            ready += (ok == 0xFFFFFFFFu) ? 32 : __ffs(~ok) - 1;
            if (ready > last) break;
            __nanosleep(100);
            if (n % 64 == 0) {
                // one lane decides, so that `ready` stays the same in every lane
                const bool expired =
                    lane == 0 && (*(volatile unsigned *)err != kErrNone || global_ns() - t0 > 1000ull * kDefaultWaitUs);
                if (__any_sync(0xFFFFFFFFu, expired)) {
                    if (lane == 0) atomicCAS(err, kErrNone, kErrTimeout);
                    ready = H;
                }
            }
        }
    };
    wait_upto(0);
    __syncthreads();
    // head: x < W unchanged, x == W -> 0
    for (int x = threadIdx.x; x <= W; x += blockDim.x) {
        const uint16_t v = (x < W) ? in[x] : (uint16_t)0;
        out[x] = v;
        ring[x & mask] = v;
    }
    const int end = N - W - 4;
    const int per = W - 1;
    // end of the staged input span of the chunk starting at sc (N % 8 == 0)
    auto span_end = [&](int sc) { return min(N, (min(sc + per, end) + W + 1 + 7) & ~7); };
    // chunk c covers [W+1 + c*per, min(+per, end)); its inputs span [s-1, e+W+1), staged from base(c)
    auto base = [&](int sc) { return (sc - 1) & ~7; };
    auto stage = [&](int sc, uint16_t *dst) {
        if (sc >= end) return;
        const int b0 = base(sc), b1 = span_end(sc);
        for (int o = threadIdx.x * 8; b0 + o < b1; o += blockDim.x * 8)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + o)),
                         "l"(in + b0 + o)
                         : "memory");
    };
    wait_upto(span_end(W + 1 + (kMedPF - 1) * per) - 1);
    __syncthreads();
    for (int c = 0; c < kMedPF; c++) {
        stage(W + 1 + c * per, bufs + (size_t)c * blen);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    int c = 0;
    for (int s = W + 1; s < end; s += per, c++) {
        asm volatile("cp.async.wait_group %0;" ::"n"(kMedPF - 1) : "memory");
        if (s + kMedPF * per < end) wait_upto(span_end(s + kMedPF * per) - 1);
        // this chunk's inputs (every thread's copies) are in, the previous chunk's outputs are in the ring,
        // the buffer of chunk c-1 is free for chunk c+kMedPF and that chunk's input rows are published
        __syncthreads();
        stage(s + kMedPF * per, bufs + (size_t)((c + kMedPF) % (kMedPF + 1)) * blen);
        asm volatile("cp.async.commit_group;" ::: "memory");
        const int e = min(s + per, end);
        const uint16_t *bi = bufs + (size_t)(c % (kMedPF + 1)) * blen - base(s); // bi[x] = in[x] for the span
        // pairs (x, x+1) at even x cover [s, e): a first pair (s-1, s) when s is odd stores only s, a last pair
        // (e-1, e) when e is odd stores only e-1 (the other half reads columns outside the chunk's inputs)
        const int s0 = s & ~1;
        const int npr = (e - s0 + 1) >> 1;
        for (int t = threadIdx.x; t * kMedPairs < npr; t += blockDim.x) {
            const int x0 = s0 + 2 * kMedPairs * t;
            // packed column words j = 0 .. kMedPairs+1 hold columns (x0 + 2j - 2, x0 + 2j - 1)
            uint32_t lo[kMedPairs + 2], mi[kMedPairs + 2], hi[kMedPairs + 2];
#pragma unroll
            for (int j = 0; j < kMedPairs + 2; j++) {
                const int cx = x0 + 2 * j - 2;
                const uint32_t top = *reinterpret_cast<const uint32_t *>(ring + ((cx - W) & mask));
                const uint32_t mid = *reinterpret_cast<const uint32_t *>(bi + cx);
                const uint32_t bot = *reinterpret_cast<const uint32_t *>(bi + cx + W);
                lo[j] = __vimin3_u16x2(top, mid, bot);
                hi[j] = __vimax3_u16x2(top, mid, bot);
                mi[j] = top + mid + bot - lo[j] - hi[j];
            }
#pragma unroll
            for (int j = 0; j < kMedPairs; j++) {
                const int x = x0 + 2 * j;
                if (x >= e) break;
                const uint32_t l3 = __vimax3_u16x2(shift1(lo[j], lo[j + 1]), lo[j + 1], shift1(lo[j + 1], lo[j + 2]));
                const uint32_t m3 = pmed3(shift1(mi[j], mi[j + 1]), mi[j + 1], shift1(mi[j + 1], mi[j + 2]));
                const uint32_t h3 = __vimin3_u16x2(shift1(hi[j], hi[j + 1]), hi[j + 1], shift1(hi[j + 1], hi[j + 2]));
                const uint32_t v = pmed3(l3, m3, h3);
                if (x >= s && x + 1 < e) {
                    *reinterpret_cast<uint32_t *>(ring + (x & mask)) = v;
                    *reinterpret_cast<uint32_t *>(out + x) = v;
                } else {
                    const int xs = x >= s ? x : x + 1;
                    const uint16_t h = (uint16_t)(x >= s ? v : v >> 16);
                    ring[xs & mask] = h;
                    out[xs] = h;
                }
            }
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    // tail: x >= N-W-4 unchanged
    wait_upto(N - 1);
    __syncthreads();
    for (int x = N - W - 4 + threadIdx.x; x < N; x += blockDim.x) out[x] = in[x];
}

// One pair per thread where the block covers a chunk's W/2 pairs in one pass (a shorter chain per chunk: the pair
// WTA + median stage of 640x480/192 0.565 -> 0.525 ms, of 640x480/128 0.44 -> 0.41 ms), else two (1920x1080/256's
// transposed maps: one pass of two pairs beats two passes of one).
__device__ __forceinline__ void median_map_any(const uint16_t *__restrict__ wta, const Geom &g, uint16_t *__restrict__ med,
                                               int k, const unsigned *rowflags, unsigned epoch, unsigned *err,
                                               uint16_t *msm) {
    const int W = g.fcols(k >> 1);
    if (W / 2 <= (int)blockDim.x)
        median_map<1>(wta, g, med, k, rowflags, epoch, err, msm);
    else
        median_map<kMedPairsMax>(wta, g, med, k, rowflags, epoch, err, msm);
}

__global__ void __launch_bounds__(1024) median_kernel(const uint16_t *__restrict__ wta, Geom g,
                                                      uint16_t *__restrict__ med, int k0, const unsigned *rowflags,
                                                      unsigned epoch, unsigned *err) {
    extern __shared__ __align__(16) uint16_t msm[];
    median_map_any(wta, g, med, k0 + blockIdx.x, rowflags, epoch, err, msm);
}

// Both WTAs of every frame row and the eight medians in one launch: blocks 0..7 sweep the medians of maps
// 0..7 and follow the rows as the other blocks publish them (row flags). The rows of the four frames are
// interleaved in proportion to their counts (frames 1 and 3 have Wp rows, frames 0 and 2 have Hp), so every
// median receives its rows at a steady rate and all eight finish close to the last row. Blocks are dispatched
// in index order in practice, so the medians start with the first rows; nothing waits on a median, so any
// dispatch order completes.
__global__ void __launch_bounds__(1024) wta_median_kernel(const uint64_t *__restrict__ census, Geom g,
                                                          uint16_t *__restrict__ wta, uint16_t *__restrict__ med,
                                                          unsigned *rowflags, unsigned epoch, unsigned *err) {
    extern __shared__ __align__(16) uint64_t fsm[];
    if (blockIdx.x < 8) {
        median_map_any(wta, g, med, blockIdx.x, rowflags, epoch, err, reinterpret_cast<uint16_t *>(fsm));
        return;
    }
    // row t of the merged sequence: A = rows of frames 1 and 3 (2 Wp), B = rows of frames 0 and 2 (2 Hp)
    const long long t = blockIdx.x - 8, na = 2LL * g.Wp, tot = na + 2LL * g.Hp;
    const long long a0 = t * na / tot, a1 = (t + 1) * na / tot; // A items before t, and up to t
    int f, i;
    if (a1 > a0) {
        f = (a0 & 1) ? 3 : 1;
        i = (int)(a0 >> 1);
    } else {
        const long long b = t - a0;
        f = (b & 1) ? 2 : 0;
        i = (int)(b >> 1);
    }
    pair_wta_row(census, g, wta, f, i, rowflags, epoch, fsm);
}

// doLRCheck(L, R, W, H, 5) (postprocess.cpp:318-341) and the mask loops of SisterMultiviewDisparities.hpp:201-251:
// keep = L <= j && |L - R[j-L]| <= 5; mask = keep && L > 0 && j >= dc; written in padded original
// coordinates (frame 2: (i, Wp-1-j); frame 1: transpose + flip(-1); frame 3: transpose + flip(1)).
// 32x32 tiles of frame coordinates (a, b); the transposed frames 1 and 3 go through a shared tile so that their
// mask rows (padded image rows i = Hp-1-b or b, columns j = Wp-1-a) are written contiguously too.
__global__ void lrc_mask_kernel(const uint16_t *__restrict__ med, Geom g, uint8_t *__restrict__ masks, int f0) {
    __shared__ uint8_t tile[32][33];
    const int f = f0 + blockIdx.z;
    const int H = g.frows(f), W = g.fcols(f);
    const int a0 = blockIdx.y * 32, b0 = blockIdx.x * 32;
    if (a0 >= H || b0 >= W) return; // block-uniform
    const int tx = threadIdx.x, ty = threadIdx.y; // 32 x 8
    uint8_t *out = masks + (size_t)f * g.plane;
    for (int s = ty; s < 32; s += 8) {
        const int a = a0 + s, b = b0 + tx;
        uint8_t m = 0;
        if (a < H && b < W) {
            const uint16_t *L = med + (size_t)(2 * f) * g.plane + (size_t)a * W;
            const uint16_t *R = med + (size_t)(2 * f + 1) * g.plane + (size_t)a * W;
            const int base = L[b];
            bool keep = false;
            if (base <= b) {
                const int diff = base - (int)R[b - base];
                keep = diff <= 5 && diff >= -5;
            }
            m = (keep && base > 0 && b >= g.dc) ? 1 : 0;
            if (!(f & 1)) out[(size_t)a * g.Wp + (f == 0 ? b : g.Wp - 1 - b)] = m;
        }
        tile[s][tx] = m;
    }
    if (f & 1) {
        __syncthreads();
        for (int s = ty; s < 32; s += 8) {
            const int b = b0 + s, a = a0 + tx; // consecutive a: consecutive (descending) columns j = Wp-1-a
            if (a < H && b < W) out[(size_t)(f == 1 ? g.Hp - 1 - b : b) * g.Wp + (g.Wp - 1 - a)] = tile[tx][s];
        }
    }
}

// doLRCheck(L, R, W, H, 5) (postprocess.cpp:318-341) as the two-view doStereo applies it (hpp:145): the left map
// keeps L where 0 <= L <= j and |L - R[j-L]| <= 5 and becomes -10 elsewhere; the right map is passed through.
// med holds the median-filtered maps of frame 0 (L, then R).
__global__ void stereo_lrc_kernel(const uint16_t *__restrict__ med, Geom g, int16_t *__restrict__ outL,
                                  uint16_t *__restrict__ outR) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= g.Wp || i >= g.Hp) return;
    const size_t p = (size_t)i * g.Wp + j;
    const uint16_t *L = med, *R = med + g.plane;
    const int base = L[p];
    bool keep = false;
    if (base <= j) {
        const int diff = base - (int)R[p - base];
        keep = diff <= 5 && diff >= -5;
    }
    outL[p] = keep ? (int16_t)base : (int16_t)-10;
    outR[p] = R[p];
}

} // namespace

void init_mask_kernels() {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, median_kernel); // its mbarriers are static shared memory
    cudaFuncSetAttribute(median_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    cudaFuncGetAttributes(&fa, wta_median_kernel);
    cudaFuncSetAttribute(wta_median_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    cudaGetLastError();
}

void launch_median(const uint16_t *wta, const Geom &g, uint16_t *med, cudaStream_t st, int f0, int nf,
                   const unsigned *rowflags, unsigned epoch, unsigned *err) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    const size_t smem = ((size_t)median_ring(mx) + (kMedPF + 1) * (2 * (size_t)mx + 32)) * sizeof(uint16_t);
    // one thread per position pair of a chunk (W/2 pairs cover its W-1 positions), up to 1024
    int threads = (mx / 2 + 31) & ~31;
    threads = threads < 64 ? 64 : threads > 1024 ? 1024 : threads;
    median_kernel<<<2 * nf, threads, smem, st>>>(wta, g, med, 2 * f0, rowflags, epoch, err);
}

void launch_wta_median(const uint64_t *census, const Geom &g, uint16_t *wta, uint16_t *med, unsigned *rowflags,
                       unsigned epoch, unsigned *err, cudaStream_t st) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    const size_t pw_smem = (size_t)mx * sizeof(uint64_t) + 2 * (size_t)mx * sizeof(uint32_t) + 32 * 32 * sizeof(uint32_t);
    const size_t md_smem = ((size_t)median_ring(mx) + (kMedPF + 1) * (2 * (size_t)mx + 32)) * sizeof(uint16_t);
    // One block size for both kinds of block. The pair WTA rows run best at two blocks per SM (512 threads at its
    // 53 registers: 1.67 ms for the rows of 1920x1080/256 against 1.93 at 640 threads, one block per SM; with the
    // neighbour row read from global memory the blocks of 4096x3000/512 fit two per SM too: 17.9 -> 17.1 ms at 512
    // threads against 1024); a median block sweeps a chunk with one or two position pairs per thread
    // (median_map_any), in as many passes as the chunk needs (three for 5120 columns, faster than two at 1024
    // threads: 4.9 against 5.3 ms for the eight medians of 4096x3000/512).
    const int threads = 512;
    const unsigned blocks = 8u + 2u * (unsigned)g.Wp + 2u * (unsigned)g.Hp;
    wta_median_kernel<<<blocks, threads, pw_smem > md_smem ? pw_smem : md_smem, st>>>(census, g, wta, med, rowflags,
                                                                                       epoch, err);
}

void launch_stereo_lrc(const uint16_t *med, const Geom &g, int16_t *outL, uint16_t *outR, cudaStream_t st) {
    stereo_lrc_kernel<<<dim3((g.Wp + 255) / 256, g.Hp), 256, 0, st>>>(med, g, outL, outR);
}

void launch_lrc_mask(const uint16_t *med, const Geom &g, uint8_t *masks, cudaStream_t st, int f0, int nf) {
    const int mx = g.Wp > g.Hp ? g.Wp : g.Hp;
    lrc_mask_kernel<<<dim3((mx + 31) / 32, (mx + 31) / 32, nf), dim3(32, 8), 0, st>>>(med, g, masks, f0);
}

} // namespace sister
