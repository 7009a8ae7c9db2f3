// Batched execution of many rigs (sister_batch_*): the throughput path for callers with many independent
// rigs at once, e.g. the 64 mixed-size rigs of one batch.
//
// One call computes every rig exactly as sister_compute would (same kernels, bit-identical outputs):
//   * rigs are packed into waves whose device memory fits the batch's budget; all device memory comes from
//     one arena allocated at sister_batch_create, carved per wave (no allocation per call);
//   * within a wave, the stages before the aggregation (upload, gray, frames, census, pair WTA + medians,
//     masks, masked costs) run per rig on a pool of streams, so the small kernels of one rig overlap with the
//     other rigs' work;
//   * the aggregation then runs as ONE persistent launch per d-stride class over the work items (rig, mode, pass,
//     band) of every job of the class, ordered by band: every CTA that draws an item finds work of some rig, so the
//     wavefront ramp of one rig (its later bands waiting for the earlier ones, ~40% of a single-rig launch) is
//     filled with other rigs' bands; a job is one (rig, mode) pair;
//   * the final winner-take-all of every job, then the output copies, follow on the main stream.
// The serving loop uses continuous admission instead (sister_engine.cu): a request must not wait for a wave.
#include "sister_gb300.h"
#include "sister_internal.h"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

using namespace sister;

namespace {

constexpr int kStreams = 16;
constexpr size_t kAlign = 256;
constexpr size_t kStagingBytes = 4u << 20; // pinned staging for item lists and rig descriptors

size_t al(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Device bytes of one rig inside a wave: prep buffers shared by its modes, plus per mode the cost, the two pass
// sums of the original image's pixels, the band hand-off records, progress counters and the output image.
struct RigBytes {
    size_t prep = 0, per_mode = 0;
};
RigBytes rig_bytes(int w, int h, int dc, int channels, int R) {
    const Geom g = make_geom(w, h, dc);
    RigBytes b;
    const size_t plane = g.plane;
    b.prep = al(channels == 3 ? 5 * (size_t)w * h * 3 : 0) + al(5 * (size_t)w * h) + al(8 * plane) +
             al(8 * plane * 8) + 2 * al(8 * plane * 2) + al(4 * plane) +
             al(4 * (size_t)std::max(g.Wp, g.Hp) * sizeof(unsigned)); // pair WTA row flags
    const size_t nbands = (size_t)(g.Hp + R - 1) / R;
    const size_t vol = plane * g.dp * 2, svol = sgm_sum_cells(g, true) * 2;
    b.per_mode = al(vol) + 2 * al(svol) + al(sgm_bnd_bytes(g, SgmPlan{})) + al(progress_bytes(2 * nbands)) +
                 al((size_t)w * h * 2);
    return b;
}

int nmodes_of(const sister_rig &r) { return (r.multi ? 1 : 0) + (r.horiz ? 1 : 0) + (r.vert ? 1 : 0); }

} // namespace

struct sister_batch {
    int device = 0;
    char *arena = nullptr;
    size_t arena_bytes = 0, top = 0;
    cudaStream_t main = nullptr;
    cudaStream_t streams[kStreams] = {};
    std::vector<cudaEvent_t> events;
    char *staging = nullptr; // pinned host
    std::string err;

    int fail(int code, const char *fmt, ...) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? SISTER_ENOMEM : SISTER_EDEVICE, "%s: %s", what,
                    cudaGetErrorString(e));
    }
    template <class T>
    T *take(size_t bytes) {
        T *p = reinterpret_cast<T *>(arena + top);
        top += al(bytes);
        return p;
    }
};

namespace {

struct Job {
    int rig, mode;
    Geom g;
    uint16_t *cost, *sum0, *sum1, *bnd, *out;
    unsigned *progress;
    int nbands;
    uint16_t *host_out;
};

int validate(sister_batch *b, const sister_rig &r, int k) {
    for (int v = 0; v < 5; v++)
        if (!r.views[v]) return b->fail(SISTER_EINVAL, "rig %d: view %d is NULL", k, v);
    if (r.channels != 1 && r.channels != 3) return b->fail(SISTER_EINVAL, "rig %d: channels must be 1 or 3", k);
    if (r.width < 4 || r.height < 4 || (r.width % 4) || (r.height % 4))
        return b->fail(SISTER_EINVAL, "rig %d: size %dx%d: width and height must be positive multiples of 4", k,
                       r.width, r.height);
    if (r.stride < r.width * r.channels) return b->fail(SISTER_EINVAL, "rig %d: stride < width*channels", k);
    if (r.max_disparity < 8 || r.max_disparity > 512 || (r.max_disparity % 8))
        return b->fail(SISTER_EINVAL, "rig %d: max disparity %d: must be a multiple of 8 in [8, 512]", k,
                       r.max_disparity);
    return SISTER_OK;
}

// Runs the rigs [first, last) as one wave; the arena has room for all of them.
int run_wave(sister_batch *b, const sister_rig *rigs, int first, int last) {
    b->top = 0;
    unsigned *errflag = b->take<unsigned>(sizeof(unsigned));
    // the rigs' streams read and raise this flag: clear it before any of them starts
    cudaError_t e = cudaMemsetAsync(errflag, 0, sizeof(unsigned), b->main);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->main);
    if (e != cudaSuccess) return b->cuda_fail(e, "reset error flag");
    std::vector<Job> jobs;
    for (int k = first; k < last; k++) {
        const sister_rig &r = rigs[k];
        if (!nmodes_of(r)) continue;
        cudaStream_t st = b->streams[(k - first) % kStreams];
        const Geom g = make_geom(r.width, r.height, r.max_disparity);
        const int w = r.width, h = r.height;
        const size_t plane = g.plane;
        // upload and gray (as sister_load_views)
        uint8_t *views = nullptr;
        const size_t row = (size_t)w * r.channels;
        uint8_t *raw = r.channels == 3 ? b->take<uint8_t>(5 * row * h) : nullptr;
        views = b->take<uint8_t>(5 * (size_t)w * h);
        if (r.channels == 1) {
            for (int v = 0; v < 5; v++) {
                e = cudaMemcpy2DAsync(views + v * (size_t)w * h, w, r.views[v], r.stride, w, h, cudaMemcpyHostToDevice, st);
                if (e != cudaSuccess) return b->cuda_fail(e, "copying views");
            }
        } else {
            const uint8_t *src[5];
            for (int v = 0; v < 5; v++) {
                e = cudaMemcpy2DAsync(raw + v * row * h, row, r.views[v], r.stride, row, h, cudaMemcpyHostToDevice, st);
                if (e != cudaSuccess) return b->cuda_fail(e, "copying views");
                src[v] = raw + v * row * h;
            }
            launch_to_gray(src, (int)row, 3, w, h, views, st);
        }
        uint8_t *frames = b->take<uint8_t>(8 * plane);
        uint64_t *census = b->take<uint64_t>(8 * plane * 8);
        uint16_t *wta = b->take<uint16_t>(8 * plane * 2);
        uint16_t *med = b->take<uint16_t>(8 * plane * 2);
        uint8_t *masks = b->take<uint8_t>(4 * plane);
        // row flags of the pair WTA / median launch: a fresh array starts at 0 and epoch 1 marks a written row
        const size_t flag_bytes = 4 * (size_t)std::max(g.Wp, g.Hp) * sizeof(unsigned);
        unsigned *rowflags = b->take<unsigned>(flag_bytes);
        e = cudaMemsetAsync(rowflags, 0, flag_bytes, st);
        if (e != cudaSuccess) return b->cuda_fail(e, "reset row flags");
        launch_frames(views, g, frames, st);
        launch_census(frames, g, census, st);
        launch_wta_median(census, g, wta, med, rowflags, 1u, errflag, st);
        launch_lrc_mask(med, g, masks, st);
        const int R = sgm_rows_max(g.dp, b->device);
        uint16_t *outs[3] = {r.multi, r.horiz, r.vert};
        for (int mode = 0; mode < 3; mode++) {
            if (!outs[mode]) continue;
            Job j{};
            j.rig = k;
            j.mode = mode;
            j.g = g;
            j.nbands = (g.Hp + R - 1) / R;
            const size_t vol = plane * g.dp * 2, svol = sgm_sum_cells(g, true) * 2;
            j.cost = b->take<uint16_t>(vol);
            j.sum0 = b->take<uint16_t>(svol);
            j.sum1 = b->take<uint16_t>(svol);
            j.bnd = b->take<uint16_t>(sgm_bnd_bytes(g, SgmPlan{}));
            j.progress = b->take<unsigned>(progress_bytes(2 * (size_t)j.nbands));
            j.out = b->take<uint16_t>((size_t)w * h * 2);
            j.host_out = outs[mode];
            launch_masked_cost(census, masks, g, mode, j.cost, st);
            e = cudaMemsetAsync(j.progress, 0, progress_bytes(2 * (size_t)j.nbands), st);
            if (e != cudaSuccess) return b->cuda_fail(e, "reset progress");
            jobs.push_back(j);
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return b->cuda_fail(e, "pre-aggregation launches");
        e = cudaEventRecord(b->events[k - first], st);
        if (e != cudaSuccess) return b->cuda_fail(e, "recording event");
        e = cudaStreamWaitEvent(b->main, b->events[k - first], 0);
        if (e != cudaSuccess) return b->cuda_fail(e, "joining streams");
    }
    // one aggregation launch per d-stride class (and per 256 jobs: the item encoding has 8 rig bits)
    size_t soff = 0;
    std::vector<int> dps;
    for (const Job &j : jobs)
        if (std::find(dps.begin(), dps.end(), j.g.dp) == dps.end()) dps.push_back(j.g.dp);
    for (int dp : dps) {
        std::vector<const Job *> cls;
        for (const Job &j : jobs)
            if (j.g.dp == dp) cls.push_back(&j);
        const int R = sgm_rows_max(dp, b->device);
        for (size_t c0 = 0; c0 < cls.size(); c0 += 256) {
            const size_t c1 = std::min(cls.size(), c0 + 256);
            // items ordered by band: every item follows the previous band of its job and pass; every job's final
            // WTA rows are placed after the bands that complete them (sgm_build_items)
            std::vector<SgmItemRig> irs;
            for (size_t q = c0; q < c1; q++) irs.push_back({cls[q]->nbands, cls[q]->g.Hp, cls[q]->g.dc, cls[q]->g.h});
            std::vector<uint32_t> items;
            sgm_build_items(irs.data(), (int)irs.size(), R, true, items);
            const size_t rig_bytes_n = (c1 - c0) * sizeof(SgmRig), item_bytes = items.size() * sizeof(uint32_t);
            if (soff + al(rig_bytes_n) + al(item_bytes) > kStagingBytes)
                return b->fail(SISTER_EBUDGET, "batch wave has too many aggregation work items (%zu)", items.size());
            SgmRig *hr = reinterpret_cast<SgmRig *>(b->staging + soff);
            uint32_t *hi = reinterpret_cast<uint32_t *>(b->staging + soff + al(rig_bytes_n));
            soff += al(rig_bytes_n) + al(item_bytes);
            for (size_t q = c0; q < c1; q++) {
                const Job &j = *cls[q];
                SgmRig &rg = hr[q - c0];
                rg.cost = j.cost;
                rg.sum0 = j.sum0;
                rg.sum1 = j.sum1;
                rg.bnd = j.bnd;
                rg.progress = j.progress;
                rg.W = j.g.Wp;
                rg.H = j.g.Hp;
                rg.D = j.g.dc;
                rg.nbands = j.nbands;
                sgm_crop_window(rg, j.g); // no padded map: the sums of the original image only
                rg.out = j.out; // the final WTA runs in the same launch
            }
            std::copy(items.begin(), items.end(), hi);
            SgmRig *dr = b->take<SgmRig>(rig_bytes_n);
            uint32_t *di = b->take<uint32_t>(item_bytes);
            unsigned *claim = b->take<unsigned>(progress_bytes(1));
            if (b->top > b->arena_bytes) return b->fail(SISTER_EBUDGET, "batch arena exhausted by descriptors");
            e = cudaMemcpyAsync(dr, hr, rig_bytes_n, cudaMemcpyHostToDevice, b->main);
            if (e == cudaSuccess) e = cudaMemcpyAsync(di, hi, item_bytes, cudaMemcpyHostToDevice, b->main);
            if (e == cudaSuccess) e = cudaMemsetAsync(claim, 0, sizeof(unsigned), b->main);
            if (e == cudaSuccess)
                e = launch_sgm_multi(dp, R, dr, di, (int)items.size(), claim, errflag, b->device, b->main);
            if (e != cudaSuccess) return b->cuda_fail(e, "aggregation launch");
        }
    }
    // the outputs (every job's final WTA ran in its aggregation launch)
    for (const Job &j : jobs) {
        const sister_rig &r = rigs[j.rig];
        e = cudaMemcpyAsync(j.host_out, j.out, (size_t)r.width * r.height * 2, cudaMemcpyDeviceToHost, b->main);
        if (e != cudaSuccess) return b->cuda_fail(e, "output copy");
    }
    unsigned flag = 0;
    e = cudaMemcpyAsync(&flag, errflag, sizeof flag, cudaMemcpyDeviceToHost, b->main);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->main);
    if (e != cudaSuccess) return b->cuda_fail(e, "batch wave");
    if (flag != kErrNone) return b->fail(SISTER_ETIMEOUT, "aggregation band hand-off wait expired (device reported timeout)");
    return SISTER_OK;
}

} // namespace

extern "C" {

size_t sister_batch_rig_bytes(int width, int height, int max_disparity, int nmodes) {
    if (width < 4 || height < 4 || max_disparity < 8 || max_disparity > 512 || nmodes < 0) return 0;
    const Geom g = make_geom(width, height, max_disparity);
    if (g.dpl < 0) return 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = -1;
    }
    const int R = dev >= 0 ? sgm_rows_max(g.dp, dev) : sgm_rows_gb300(g.dp);
    const RigBytes rb = rig_bytes(width, height, max_disparity, 3, R);
    return rb.prep + (size_t)nmodes * rb.per_mode;
}

int sister_batch_create(sister_batch **out, int device, size_t budget_bytes) {
    if (!out) return SISTER_EINVAL;
    *out = nullptr;
    sister_batch *b = new sister_batch();
    b->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        cudaGetLastError();
        delete b;
        return SISTER_EDEVICE;
    }
    init_mask_kernels();
    init_sgm_kernels();
    if (!budget_bytes) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget_bytes = fr / 4 * 3;
    }
    b->arena_bytes = budget_bytes & ~(kAlign - 1);
    e = cudaMalloc(&b->arena, b->arena_bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->main, cudaStreamNonBlocking);
    for (int s = 0; s < kStreams && e == cudaSuccess; s++) e = cudaStreamCreateWithFlags(&b->streams[s], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMallocHost(&b->staging, kStagingBytes);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? SISTER_ENOMEM : SISTER_EDEVICE;
        cudaGetLastError();
        sister_batch_destroy(b);
        return code;
    }
    *out = b;
    return SISTER_OK;
}

void sister_batch_destroy(sister_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->main) cudaStreamSynchronize(b->main);
    for (cudaStream_t s : b->streams)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    if (b->main) cudaStreamDestroy(b->main);
    for (cudaEvent_t ev : b->events) cudaEventDestroy(ev);
    if (b->arena) cudaFree(b->arena);
    if (b->staging) cudaFreeHost(b->staging);
    cudaGetLastError();
    delete b;
}

const char *sister_batch_last_error(sister_batch *b) { return b ? b->err.c_str() : "null batch"; }

int sister_batch_run(sister_batch *b, const sister_rig *rigs, int nrigs) {
    if (!b) return SISTER_EINVAL;
    if (nrigs < 0 || (nrigs > 0 && !rigs)) return b->fail(SISTER_EINVAL, "rigs is NULL");
    cudaSetDevice(b->device);
    std::vector<size_t> need(nrigs);
    for (int k = 0; k < nrigs; k++) {
        int rc = validate(b, rigs[k], k);
        if (rc) return rc;
        const Geom g = make_geom(rigs[k].width, rigs[k].height, rigs[k].max_disparity);
        const RigBytes rb = rig_bytes(rigs[k].width, rigs[k].height, rigs[k].max_disparity, rigs[k].channels,
                                      sgm_rows_max(g.dp, b->device));
        need[k] = rb.prep + nmodes_of(rigs[k]) * rb.per_mode;
        if (need[k] + kAlign + 2 * kStagingBytes > b->arena_bytes)
            return b->fail(SISTER_EBUDGET, "rig %d (%dx%d, max disparity %d) needs %zu bytes; the batch budget is %zu", k,
                           rigs[k].width, rigs[k].height, rigs[k].max_disparity, need[k], b->arena_bytes);
    }
    // waves: consecutive rigs while they fit (with slack for descriptors), at most 256 rigs each
    int first = 0;
    while (first < nrigs) {
        size_t used = kAlign + 2 * kStagingBytes;
        int last = first;
        while (last < nrigs && last - first < 256 && used + need[last] <= b->arena_bytes) used += need[last++];
        if ((int)b->events.size() < last - first) {
            const size_t old = b->events.size();
            b->events.resize(last - first);
            for (size_t q = old; q < b->events.size(); q++) {
                cudaError_t e = cudaEventCreateWithFlags(&b->events[q], cudaEventDisableTiming);
                if (e != cudaSuccess) return b->cuda_fail(e, "creating events");
            }
        }
        int rc = run_wave(b, rigs, first, last);
        if (rc) return rc;
        first = last;
    }
    return SISTER_OK;
}

} // extern "C"
