// Host runtime of libsister_gb300: context, device buffers, stage orchestration and the C ABI of
// include/sister_gb300.h.
#include "sister_gb300.h"
#include "sister_internal.h"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace sister;

namespace {

struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        release();
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            return e;
        }
        cap = bytes;
        return cudaSuccess;
    }
    template <typename T> T *as() const { return reinterpret_cast<T *>(p); }
};

std::mutex g_init_mu;
std::vector<int> g_inited_devices;

void init_device_kernels(int dev) {
    std::lock_guard<std::mutex> lk(g_init_mu);
    for (int d : g_inited_devices)
        if (d == dev) return;
    init_mask_kernels();
    init_sgm_kernels();
    g_inited_devices.push_back(dev);
}

} // namespace

struct sister_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    bool loaded = false;
    int w = 0, h = 0, dc = 0;
    DevBuf raw, views, frames, census, wta, med, masks, cost, sum0, sum1, bnd, progress, errflag, disp, outs;
    // several modes in one call: per extra mode its own cost, sum and hand-off buffers, and the device descriptors
    // (rigs, work items, item ticket) of one multi-job aggregation launch
    DevBuf modevols, desc;
    int desc_key[4] = {0, 0, 0, 0}; // w, h, dc, mode mask the descriptors were built for
    SgmRig desc_rigs[3] = {};        // and the buffers they point to
    // pair WTA row flags: [4][max(Wp, Hp)] u32 holding the epoch (compute count) in which the row was written
    DevBuf rowflags;
    unsigned epoch = 0;
    SgmPlan plan{};
    int plan_w = 0, plan_h = 0, plan_dc = 0;
    int tune_rows = 0, tune_cs = 0;
    bool full_disp = false; // keep the padded disparity map (debug inspection)
    unsigned wait_limit_us = kDefaultWaitUs; // limit of every device-side wait on another warp or CTA
    // stage profiling: events recorded on the context stream around every stage of a compute
    bool prof = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int> ev_stage; // stage id that ends at event k (k >= 1)
    void mark(int stage) {
        if (!prof) return;
        if (ev.size() <= ev_stage.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            ev.push_back(e);
        }
        cudaEventRecord(ev[ev_stage.size()], stream);
        ev_stage.push_back(stage);
    }
    int last_mode = -1;
    const uint16_t *last_cost = nullptr, *last_sum0 = nullptr; // volumes of the last aggregated mode
    bool last_cropped = false; // whether last_sum0 holds only the original image's pixels
    bool have_intermediates = false;
    Geom g{};

    int fail(int code, const char *fmt, ...) __attribute__((format(printf, 3, 4))) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        err = buf;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *what) {
        cudaGetLastError();
        if (e == cudaErrorMemoryAllocation) return fail(SISTER_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
        return fail(SISTER_EDEVICE, "%s: %s", what, cudaGetErrorString(e));
    }
};

namespace {

int check_geometry(sister_ctx *c, int w, int h, int dc) {
    if (w < 4 || h < 4 || (w % 4) || (h % 4))
        return c->fail(SISTER_EINVAL, "image size %dx%d: width and height must be positive multiples of 4", w, h);
    if (dc < 8 || dc > 512 || (dc % 8))
        return c->fail(SISTER_EINVAL, "max disparity %d: must be a multiple of 8 in [8, 512]", dc);
    return SISTER_OK;
}

int load_common(sister_ctx *c, const uint8_t *const views[5], int width, int height, int stride, int channels,
                bool device_ptrs) {
    if (!views) return c->fail(SISTER_EINVAL, "views is NULL");
    for (int k = 0; k < 5; k++)
        if (!views[k]) return c->fail(SISTER_EINVAL, "view %d is NULL", k);
    if (channels != 1 && channels != 3) return c->fail(SISTER_EINVAL, "channels must be 1 or 3, got %d", channels);
    if (width < 4 || height < 4 || (width % 4) || (height % 4))
        return c->fail(SISTER_EINVAL, "image size %dx%d: width and height must be positive multiples of 4", width,
                       height);
    if (stride < width * channels) return c->fail(SISTER_EINVAL, "stride %d < width*channels", stride);
    cudaSetDevice(c->device);
    const size_t plane = (size_t)width * height;
    cudaError_t e = c->views.ensure(5 * plane);
    if (e != cudaSuccess) return c->cuda_fail(e, "allocating views");
    const uint8_t *src[5];
    if (device_ptrs) {
        for (int k = 0; k < 5; k++) src[k] = views[k];
        launch_to_gray(src, stride, channels, width, height, c->views.as<uint8_t>(), c->stream);
    } else {
        const size_t row = (size_t)width * channels;
        if (channels == 1) {
            for (int k = 0; k < 5; k++) {
                e = cudaMemcpy2DAsync(c->views.as<uint8_t>() + k * plane, width, views[k], stride, width, height,
                                      cudaMemcpyHostToDevice, c->stream);
                if (e != cudaSuccess) return c->cuda_fail(e, "copying views");
            }
        } else {
            e = c->raw.ensure(5 * row * height);
            if (e != cudaSuccess) return c->cuda_fail(e, "allocating raw views");
            for (int k = 0; k < 5; k++) {
                e = cudaMemcpy2DAsync(c->raw.as<uint8_t>() + k * row * height, row, views[k], stride, row, height,
                                      cudaMemcpyHostToDevice, c->stream);
                if (e != cudaSuccess) return c->cuda_fail(e, "copying views");
                src[k] = c->raw.as<uint8_t>() + k * row * height;
            }
            launch_to_gray(src, (int)row, 3, width, height, c->views.as<uint8_t>(), c->stream);
        }
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return c->cuda_fail(e, "loading views");
    c->w = width;
    c->h = height;
    c->loaded = true;
    c->have_intermediates = false;
    return SISTER_OK;
}

const SgmPlan &plan_for(sister_ctx *c, const Geom &g) {
    if (c->plan_w != g.w || c->plan_h != g.h || c->plan_dc != g.dc) {
        c->plan = sgm_plan(g, c->device, c->tune_rows, c->tune_cs);
        c->plan_w = g.w;
        c->plan_h = g.h;
        c->plan_dc = g.dc;
    }
    return c->plan;
}

int ensure_buffers(sister_ctx *c, const Geom &g) {
    const size_t plane = g.plane, vol = plane * g.dp;
    const SgmPlan &p = plan_for(c, g);
    if (p.R < 1) return c->fail(SISTER_EDEVICE, "no launch configuration fits the aggregation kernel");
    struct {
        DevBuf *b;
        size_t bytes;
        const char *what;
    } req[] = {
        {&c->frames, 8 * plane, "frames"},
        {&c->census, 8 * plane * sizeof(uint64_t), "census"},
        {&c->wta, 8 * plane * sizeof(uint16_t), "wta"},
        {&c->med, 8 * plane * sizeof(uint16_t), "median"},
        {&c->masks, 4 * plane, "masks"},
        {&c->cost, vol * sizeof(uint16_t), "cost volume"},
        {&c->sum0, sgm_sum_cells(g, !c->full_disp) * sizeof(uint16_t), "pass-0 sum volume"},
        {&c->sum1, sgm_sum_cells(g, !c->full_disp) * sizeof(uint16_t), "pass-1 sum volume"},
        {&c->bnd, sgm_bnd_bytes(g, p), "band boundary states"},
        {&c->progress, sgm_progress_bytes(std::max(p.ngroups, 1)), "progress"},
        {&c->errflag, sizeof(unsigned), "error flag"},
        {&c->disp, (c->full_disp ? 3 * plane : 1) * sizeof(uint16_t), "disparity"},
        {&c->outs, 3 * (size_t)g.w * g.h * sizeof(uint16_t), "outputs"},
    };
    for (auto &r : req) {
        cudaError_t e = r.b->ensure(r.bytes);
        if (e != cudaSuccess) return c->cuda_fail(e, r.what);
    }
    // a new flag array starts at 0, which no epoch takes
    void *old = c->rowflags.p;
    cudaError_t e = c->rowflags.ensure(4 * (size_t)std::max(g.Wp, g.Hp) * sizeof(unsigned));
    if (e == cudaSuccess && c->rowflags.p != old) e = cudaMemsetAsync(c->rowflags.p, 0, c->rowflags.cap, c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "row flags");
    return SISTER_OK;
}

// The requested modes of one rig (the reference's compute_disparities computes all three, hpp:77-89): each mode's
// masked cost into its own volume, then ONE aggregation launch over the work items of every mode (band items
// ordered by band, so each follows the previous band of its mode and pass; without the padded map each mode's
// final WTA rows follow as work items of the same launch, see sgm_build_items). One launch instead of one per mode:
// the wavefront ramp and tail of each mode are filled by the other modes' bands and by the WTA rows.
int run_modes_together(sister_ctx *c, const Geom &g, const SgmPlan &plan, uint16_t *dev_out[3]) {
    cudaStream_t st = c->stream;
    int modes[3], nm = 0, mask = 0;
    for (int m = 0; m < 3; m++)
        if (dev_out[m]) {
            modes[nm++] = m;
            mask |= 1 << m;
        }
    const bool cropped = !c->full_disp; // the pass sums of the original image only, unless the padded map is kept
    const bool fuse = cropped; // the final WTA as work items of the aggregation launch (the padded map: its own kernel)
    const size_t vol = g.plane * g.dp * sizeof(uint16_t), svol = sgm_sum_cells(g, cropped) * sizeof(uint16_t);
    const size_t bnd = sgm_bnd_bytes(g, plan), prog = sgm_progress_bytes(std::max(plan.ngroups, 1));
    const size_t per = vol + 2 * svol + bnd + prog; // cost, sum0, sum1, hand-off records, progress counters
    cudaError_t e = c->modevols.ensure((size_t)(nm - 1) * per);
    if (e != cudaSuccess) return c->cuda_fail(e, "per-mode volumes");
    SgmRig rg[3];
    std::memset(rg, 0, sizeof rg);
    for (int k = 0; k < nm; k++) {
        SgmRig &a = rg[k];
        if (k == 0) {
            a.cost = c->cost.as<uint16_t>();
            a.sum0 = c->sum0.as<uint16_t>();
            a.sum1 = c->sum1.as<uint16_t>();
            a.bnd = c->bnd.as<uint16_t>();
            a.progress = c->progress.as<unsigned>();
        } else {
            char *b = c->modevols.as<char>() + (size_t)(k - 1) * per;
            a.cost = reinterpret_cast<uint16_t *>(b);
            a.sum0 = reinterpret_cast<uint16_t *>(b + vol);
            a.sum1 = reinterpret_cast<uint16_t *>(b + vol + svol);
            a.bnd = reinterpret_cast<uint16_t *>(b + vol + 2 * svol);
            a.progress = reinterpret_cast<unsigned *>(b + vol + 2 * svol + bnd);
        }
        a.W = g.Wp;
        a.H = g.Hp;
        a.D = g.dc;
        a.nbands = plan.nbands;
        if (cropped) sgm_crop_window(a, g);
        if (fuse) a.out = dev_out[modes[k]];
    }
    std::vector<uint32_t> items;
    {
        const SgmItemRig ir{plan.nbands, g.Hp, g.dc, g.h};
        const SgmItemRig irs[3] = {ir, ir, ir};
        sgm_build_items(irs, nm, plan.R, fuse, items);
    }
    const int nitems = (int)items.size();
    const size_t rig_bytes = 3 * sizeof(SgmRig), item_off = (rig_bytes + 255) & ~(size_t)255;
    const size_t claim_off = (item_off + (size_t)nitems * 4 + 255) & ~(size_t)255;
    e = c->desc.ensure(claim_off + progress_bytes(1));
    if (e != cudaSuccess) return c->cuda_fail(e, "aggregation descriptors");
    char *desc = c->desc.as<char>();
    if (c->desc_key[0] != g.w || c->desc_key[1] != g.h || c->desc_key[2] != g.dc || c->desc_key[3] != mask ||
        std::memcmp(c->desc_rigs, rg, (size_t)nm * sizeof(SgmRig)) != 0) {
        e = cudaMemcpyAsync(desc, rg, rig_bytes, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(desc + item_off, items.data(), items.size() * 4, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st); // the host vectors go out of scope
        if (e != cudaSuccess) return c->cuda_fail(e, "aggregation descriptors");
        c->desc_key[0] = g.w;
        c->desc_key[1] = g.h;
        c->desc_key[2] = g.dc;
        c->desc_key[3] = mask;
        std::memcpy(c->desc_rigs, rg, (size_t)nm * sizeof(SgmRig));
    }
    for (int k = 0; k < nm; k++) {
        launch_masked_cost(c->census.as<uint64_t>(), c->masks.as<uint8_t>(), g, modes[k], const_cast<uint16_t *>(rg[k].cost),
                           st);
        e = cudaMemsetAsync(rg[k].progress, 0, prog, st);
        if (e != cudaSuccess) return c->cuda_fail(e, "progress counters");
    }
    c->mark(SISTER_STAGE_COST);
    e = cudaMemsetAsync(desc + claim_off, 0, sizeof(unsigned), st);
    if (e == cudaSuccess)
        e = launch_sgm_multi(g.dp, plan.R, reinterpret_cast<const SgmRig *>(desc),
                             reinterpret_cast<const uint32_t *>(desc + item_off), nitems,
                             reinterpret_cast<unsigned *>(desc + claim_off), c->errflag.as<unsigned>(), c->device, st,
                             c->wait_limit_us);
    if (e != cudaSuccess) return c->cuda_fail(e, "aggregation launch");
    c->mark(SISTER_STAGE_AGGREGATE);
    if (!fuse)
        for (int k = 0; k < nm; k++) {
            e = launch_sgm_wta(g, rg[k].sum0, rg[k].sum1, dev_out[modes[k]],
                               cropped ? nullptr : c->disp.as<uint16_t>() + (size_t)modes[k] * g.plane, st, cropped);
            if (e != cudaSuccess) return c->cuda_fail(e, "winner-take-all launch");
        }
    c->mark(SISTER_STAGE_WTA);
    c->last_mode = modes[nm - 1];
    c->last_cost = rg[nm - 1].cost;
    c->last_sum0 = rg[nm - 1].sum0;
    c->last_cropped = cropped;
    c->have_intermediates = true;
    return SISTER_OK;
}

// The whole compute_disparities pipeline on the context stream; outputs (device) may be null.
int run_pipeline(sister_ctx *c, uint16_t *dev_out[3]) {
    if (!c->loaded) return c->fail(SISTER_ESTATE, "no views loaded");
    if (!c->dc) return c->fail(SISTER_ESTATE, "max disparity not set");
    int rc = check_geometry(c, c->w, c->h, c->dc);
    if (rc) return rc;
    cudaSetDevice(c->device);
    const Geom g = make_geom(c->w, c->h, c->dc);
    rc = ensure_buffers(c, g);
    if (rc) return rc;
    c->g = g;
    cudaStream_t st = c->stream;
    cudaError_t e = cudaMemsetAsync(c->errflag.p, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return c->cuda_fail(e, "reset error flag");
    c->ev_stage.clear();
    c->mark(-1);
    launch_frames(c->views.as<uint8_t>(), g, c->frames.as<uint8_t>(), st);
    c->mark(SISTER_STAGE_FRAMES);
    launch_census(c->frames.as<uint8_t>(), g, c->census.as<uint64_t>(), st);
    c->mark(SISTER_STAGE_CENSUS);
    // Pair WTA of the four frames and the eight medians in one launch: the median blocks come first and follow
    // the WTA rows as they are published (each row with this compute's epoch); the masks follow. With
    // profiling on, the pair WTA stage covers that launch.
    if (++c->epoch == 0) c->epoch = 1;
    launch_wta_median(c->census.as<uint64_t>(), g, c->wta.as<uint16_t>(), c->med.as<uint16_t>(),
                      c->rowflags.as<unsigned>(), c->epoch, c->errflag.as<unsigned>(), st);
    c->mark(SISTER_STAGE_PAIR_WTA);
    launch_lrc_mask(c->med.as<uint16_t>(), g, c->masks.as<uint8_t>(), st);
    c->mark(SISTER_STAGE_MASKS);
    e = cudaGetLastError();
    if (e != cudaSuccess) return c->cuda_fail(e, "mask stage launch");
    const SgmPlan &plan = plan_for(c, g);
    const int nmodes = (dev_out[0] ? 1 : 0) + (dev_out[1] ? 1 : 0) + (dev_out[2] ? 1 : 0);
    if (nmodes == 0) { // nothing to aggregate: the mask-stage intermediates are still available for inspection
        c->have_intermediates = true;
        return SISTER_OK;
    }
    // one aggregation launch for every requested output (each mode's cost into its own volume)
    return run_modes_together(c, g, plan, dev_out);
}

int read_device_error(sister_ctx *c) {
    unsigned flag = 0;
    cudaError_t e = cudaMemcpy(&flag, c->errflag.p, sizeof flag, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return c->cuda_fail(e, "reading device error flag");
    if (flag == kErrTimeout)
        return c->fail(SISTER_ETIMEOUT, "a bounded device wait expired (aggregation band hand-off or median row "
                                        "flags; device reported timeout)");
    return SISTER_OK;
}

} // namespace

extern "C" {

int sister_ctx_create(sister_ctx **out, int device) {
    if (!out) return SISTER_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
        cudaGetLastError();
        return SISTER_EDEVICE;
    }
    sister_ctx *c = new (std::nothrow) sister_ctx();
    if (!c) return SISTER_ENOMEM;
    c->device = device;
    cudaSetDevice(device);
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (!coop || cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return SISTER_EDEVICE;
    }
    c->stream = c->own_stream;
    init_device_kernels(device);
    if (c->errflag.ensure(sizeof(unsigned)) != cudaSuccess) {
        delete c;
        return SISTER_ENOMEM;
    }
    *out = c;
    return SISTER_OK;
}

void sister_ctx_destroy(sister_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    for (cudaEvent_t e : c->ev) cudaEventDestroy(e);
    if (c->own_stream) {
        cudaStreamSynchronize(c->own_stream);
        cudaStreamDestroy(c->own_stream);
    }
    delete c;
}

const char *sister_last_error(const sister_ctx *c) { return c ? c->err.c_str() : "null context"; }

int sister_load_views(sister_ctx *c, const uint8_t *const views[5], int width, int height, int stride,
                      int channels) {
    if (!c) return SISTER_EINVAL;
    return load_common(c, views, width, height, stride, channels, false);
}

int sister_load_views_device(sister_ctx *c, const uint8_t *const views[5], int width, int height, int stride,
                             int channels) {
    if (!c) return SISTER_EINVAL;
    return load_common(c, views, width, height, stride, channels, true);
}

int sister_set_max_disparity(sister_ctx *c, int dc) {
    if (!c) return SISTER_EINVAL;
    if (dc < 8 || dc > 512 || (dc % 8))
        return c->fail(SISTER_EINVAL, "max disparity %d: must be a multiple of 8 in [8, 512]", dc);
    c->dc = dc;
    return SISTER_OK;
}

int sister_compute_device(sister_ctx *c, uint16_t *multi, uint16_t *horiz, uint16_t *vert) {
    if (!c) return SISTER_EINVAL;
    uint16_t *o[3] = {multi, horiz, vert};
    return run_pipeline(c, o);
}

int sister_compute(sister_ctx *c, uint16_t *multi, uint16_t *horiz, uint16_t *vert) {
    if (!c) return SISTER_EINVAL;
    if (!c->loaded) return c->fail(SISTER_ESTATE, "no views loaded");
    if (!c->dc) return c->fail(SISTER_ESTATE, "max disparity not set");
    int rc = check_geometry(c, c->w, c->h, c->dc);
    if (rc) return rc;
    cudaSetDevice(c->device);
    rc = ensure_buffers(c, make_geom(c->w, c->h, c->dc));
    if (rc) return rc;
    const size_t n = (size_t)c->w * c->h;
    uint16_t *host[3] = {multi, horiz, vert};
    uint16_t *dev[3];
    for (int m = 0; m < 3; m++) dev[m] = host[m] ? c->outs.as<uint16_t>() + (size_t)m * n : nullptr;
    rc = run_pipeline(c, dev);
    if (rc) return rc;
    for (int m = 0; m < 3; m++) {
        if (!host[m]) continue;
        cudaError_t e = cudaMemcpyAsync(host[m], dev[m], n * sizeof(uint16_t), cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess) return c->cuda_fail(e, "copying result");
    }
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "compute");
    return read_device_error(c);
}

int sister_stereo(sister_ctx *c, const uint8_t *center, const uint8_t *other, int width, int height, int stride,
                  int dc, int16_t *left, uint16_t *right) {
    if (!c) return SISTER_EINVAL;
    if (!center || !other || !left || !right) return c->fail(SISTER_EINVAL, "stereo: NULL image or output");
    int rc = check_geometry(c, width, height, dc);
    if (rc) return rc;
    if (stride < width) return c->fail(SISTER_EINVAL, "stride %d < width", stride);
    cudaSetDevice(c->device);
    // doStereo works on the images as given (no padding): frame 0 of a geometry whose padded size is the image
    Geom g{};
    g.w = width;
    g.h = height;
    g.dc = dc;
    g.Wp = width;
    g.Hp = height;
    g.dpl = choose_dpl(dc);
    g.dp = 32 * g.dpl;
    g.plane = (size_t)width * height;
    const SgmPlan p = sgm_plan(g, c->device);
    if (p.R < 1) return c->fail(SISTER_EDEVICE, "no launch configuration fits the aggregation kernel");
    const size_t plane = g.plane, vol = plane * g.dp;
    struct {
        DevBuf *b;
        size_t bytes;
        const char *what;
    } req[] = {
        {&c->frames, 2 * plane, "frames"},
        {&c->census, 2 * plane * sizeof(uint64_t), "census"},
        {&c->wta, 2 * plane * sizeof(uint16_t), "wta"},
        {&c->med, 2 * plane * sizeof(uint16_t), "median"},
        {&c->cost, vol * sizeof(uint16_t), "cost volume"},
        {&c->sum0, vol * sizeof(uint16_t), "pass-0 sum volume"},
        {&c->sum1, vol * sizeof(uint16_t), "pass-1 sum volume"},
        {&c->bnd, sgm_bnd_bytes(g, p), "band boundary states"},
        {&c->progress, sgm_progress_bytes(std::max(p.ngroups, 1)), "progress"},
        {&c->outs, 2 * plane * sizeof(uint16_t), "outputs"},
    };
    for (auto &r : req) {
        cudaError_t e = r.b->ensure(r.bytes);
        if (e != cudaSuccess) return c->cuda_fail(e, r.what);
    }
    c->have_intermediates = false; // the multiview intermediates are overwritten
    cudaStream_t st = c->stream;
    uint8_t *frames = c->frames.as<uint8_t>();
    cudaError_t e = cudaMemsetAsync(c->errflag.p, 0, sizeof(unsigned), st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(frames, width, center, stride, width, height, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(frames + plane, width, other, stride, width, height, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return c->cuda_fail(e, "copying images");
    // ad_census (hpp:135): census of both images, Hamming volume (frame 0 alone, unmasked)
    launch_census(frames, g, c->census.as<uint64_t>(), st, 2);
    launch_masked_cost(c->census.as<uint64_t>(), nullptr, g, 3, c->cost.as<uint16_t>(), st);
    // sgm (hpp:138)
    SgmRig a{};
    a.cost = c->cost.as<uint16_t>();
    a.sum0 = c->sum0.as<uint16_t>();
    a.sum1 = c->sum1.as<uint16_t>();
    a.bnd = c->bnd.as<uint16_t>();
    a.progress = c->progress.as<unsigned>();
    e = launch_sgm(g, p, a, c->errflag.as<unsigned>(), st, c->wait_limit_us);
    if (e != cudaSuccess) return c->cuda_fail(e, "aggregation launch");
    // WTALeft / WTARight (hpp:141-142) into maps 0 and 1 of frame 0, their in-place medians (hpp:143-144), LR check
    uint16_t *wta = c->wta.as<uint16_t>();
    e = launch_sgm_wta(g, a.sum0, a.sum1, nullptr, wta, st, false); // the whole plane: WTARight reads its diagonals
    if (e == cudaSuccess) e = launch_sgm_wta_right(g, a.sum0, a.sum1, wta + plane, st);
    if (e != cudaSuccess) return c->cuda_fail(e, "winner-take-all launch");
    launch_median(wta, g, c->med.as<uint16_t>(), st, 0, 1);
    int16_t *dl = c->outs.as<int16_t>();
    uint16_t *dr = c->outs.as<uint16_t>() + plane;
    launch_stereo_lrc(c->med.as<uint16_t>(), g, dl, dr, st);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(left, dl, plane * sizeof(int16_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(right, dr, plane * sizeof(uint16_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c->cuda_fail(e, "stereo");
    return read_device_error(c);
}

int sister_set_stream(sister_ctx *c, void *stream) {
    if (!c) return SISTER_EINVAL;
    c->stream = stream ? (cudaStream_t)stream : c->own_stream;
    return SISTER_OK;
}

int sister_synchronize(sister_ctx *c) {
    if (!c) return SISTER_EINVAL;
    cudaSetDevice(c->device);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "synchronize");
    return read_device_error(c);
}

size_t sister_device_bytes(int width, int height, int dc) {
    if (width <= 0 || height <= 0 || dc <= 0) return 0;
    const Geom g = make_geom(width, height, dc);
    if (g.dpl < 0) return 0;
    const size_t plane = g.plane, vol = plane * g.dp;
    // band boundary records: one image row per band and pass, with the band height the launch plan picks on
    // the current device (or a 152-SM GB300 when there is none), progress counters, sum volumes of both passes
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        dev = -1;
    }
    SgmPlan p{};
    if (dev >= 0) {
        init_sgm_kernels();
        p = sgm_plan(g, dev);
    }
    if (p.R < 1) p = sgm_plan_gb300(g);
    if (p.R < 1) return 0;
    const size_t nbands = (size_t)p.nbands;
    const size_t bnd = sgm_bnd_bytes(g, p);
    // one compute of one mode without the padded map: the cost volume and two pass sums of the original image
    return 5 * (size_t)width * height + 8 * plane + 8 * plane * 8 + 2 * 8 * plane * 2 + 4 * plane + vol * 2 +
           2 * sgm_sum_cells(g, true) * 2 + bnd + sgm_progress_bytes(2 * nbands) + 2 + 3 * (size_t)width * height * 2;
}

int sister_profile_enable(sister_ctx *c, int on) {
    if (!c) return SISTER_EINVAL;
    c->prof = on != 0;
    c->ev_stage.clear();
    return SISTER_OK;
}

int sister_profile_read(sister_ctx *c, float *ms, int *stage, int max, int *count) {
    if (!c || !count) return SISTER_EINVAL;
    *count = 0;
    if (!c->prof || c->ev_stage.size() < 2) return SISTER_OK;
    cudaSetDevice(c->device);
    cudaError_t e = cudaEventSynchronize(c->ev[c->ev_stage.size() - 1]);
    if (e != cudaSuccess) return c->cuda_fail(e, "profile read");
    int n = 0;
    for (size_t k = 1; k < c->ev_stage.size() && n < max; k++, n++) {
        float t = 0;
        cudaEventElapsedTime(&t, c->ev[k - 1], c->ev[k]);
        if (ms) ms[n] = t;
        if (stage) stage[n] = c->ev_stage[k];
    }
    *count = n;
    return SISTER_OK;
}

int sister_tune_set(sister_ctx *c, int key, int value) {
    if (!c) return SISTER_EINVAL;
    switch (key) {
    case SISTER_TUNE_SGM_ROWS:
        if (value < 0 || value > 16) return c->fail(SISTER_EINVAL, "rows per CTA must be in [0, 16]");
        c->tune_rows = value;
        break;
    case SISTER_TUNE_SGM_CLUSTER:
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8)
            return c->fail(SISTER_EINVAL, "cluster size must be 0, 1, 2, 4 or 8");
        c->tune_cs = value;
        break;
    case SISTER_TUNE_FULL_DISP: c->full_disp = value != 0; return SISTER_OK;
    case SISTER_TUNE_WAIT_LIMIT_US:
        if (value < 0) return c->fail(SISTER_EINVAL, "wait limit must be >= 0 microseconds (0: default)");
        c->wait_limit_us = value ? (unsigned)value : kDefaultWaitUs;
        return SISTER_OK;
    default: return c->fail(SISTER_EINVAL, "unknown or read-only tuning key %d", key);
    }
    c->plan_w = c->plan_h = c->plan_dc = 0; // re-plan on next use
    return SISTER_OK;
}

int sister_tune_get(sister_ctx *c, int key, int *value) {
    if (!c || !value) return SISTER_EINVAL;
    if (!c->loaded || !c->dc) return c->fail(SISTER_ESTATE, "load views and set the max disparity first");
    cudaSetDevice(c->device);
    const SgmPlan &p = plan_for(c, make_geom(c->w, c->h, c->dc));
    switch (key) {
    case SISTER_TUNE_SGM_ROWS: *value = p.R; break;
    case SISTER_TUNE_SGM_CLUSTER: *value = p.cs; break;
    case SISTER_TUNE_SGM_GROUPS: *value = p.ngroups; break;
    case SISTER_TUNE_SGM_CLUSTERS: *value = p.nclusters; break;
    case SISTER_TUNE_FULL_DISP: *value = c->full_disp ? 1 : 0; break;
    case SISTER_TUNE_WAIT_LIMIT_US: *value = (int)c->wait_limit_us; break;
    default: return c->fail(SISTER_EINVAL, "unknown tuning key %d", key);
    }
    return SISTER_OK;
}

int sister_debug_fetch(sister_ctx *c, int what, int index, void *dst, size_t bytes) {
    if (!c || !dst) return SISTER_EINVAL;
    if (what == SISTER_DBG_DP) {
        if (bytes < sizeof(int)) return SISTER_EINVAL;
        *(int *)dst = c->g.dp;
        return SISTER_OK;
    }
    if (!c->have_intermediates) return c->fail(SISTER_ESTATE, "no computation to inspect");
    cudaSetDevice(c->device);
    const Geom &g = c->g;
    const size_t plane = g.plane;
    const char *src = nullptr;
    size_t need = 0;
    switch (what) {
    case SISTER_DBG_FRAMES: src = c->frames.as<char>() + (size_t)index * plane; need = plane; break;
    case SISTER_DBG_CENSUS: src = c->census.as<char>() + (size_t)index * plane * 8; need = plane * 8; break;
    case SISTER_DBG_WTA: src = c->wta.as<char>() + (size_t)index * plane * 2; need = plane * 2; break;
    case SISTER_DBG_MEDIAN: src = c->med.as<char>() + (size_t)index * plane * 2; need = plane * 2; break;
    case SISTER_DBG_MASKS: src = c->masks.as<char>() + (size_t)index * plane; need = plane; break;
    case SISTER_DBG_COST: src = reinterpret_cast<const char *>(c->last_cost); need = plane * g.dp * 2; break;
    case SISTER_DBG_SUM0:
        if (c->last_cropped)
            return c->fail(SISTER_ESTATE, "the whole pass-0 sum volume is kept only with SISTER_TUNE_FULL_DISP = 1");
        src = reinterpret_cast<const char *>(c->last_sum0);
        need = plane * g.dp * 2;
        break;
    case SISTER_DBG_DISP:
        if (!c->full_disp) return c->fail(SISTER_ESTATE, "the padded disparity map is kept only with SISTER_TUNE_FULL_DISP = 1");
        src = c->disp.as<char>() + (size_t)index * plane * 2;
        need = plane * 2;
        break;
    default: return c->fail(SISTER_EINVAL, "unknown debug item %d", what);
    }
    if (index < 0 || index > 7 || bytes < need) return c->fail(SISTER_EINVAL, "bad debug index/size");
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(dst, src, need, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return c->cuda_fail(e, "debug fetch");
    return SISTER_OK;
}

} // extern "C"
