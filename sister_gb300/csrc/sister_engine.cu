// Request engine of the serving loop: continuous admission of independent rigs (requests).
//
// A request is admitted as soon as a stream slot is free and its device memory fits the budget next to the
// rigs already admitted -- not when an earlier group of requests has finished. Each admitted rig then runs the
// whole pipeline of sister_compute on its own stream: upload, gray, frames, census, pair WTA + medians, masks,
// and per requested mode the masked cost, the aggregation and the final WTA, then the output download. Rigs on
// different streams overlap on the device: one rig's stages fill the SMs another rig's kernels leave (the
// aggregation of a small rig occupies a few dozen SMs; any rig's ramp and tail leave SMs idle). Memory comes
// from a dedicated stream-ordered pool (allocated at admission, freed on the rig's stream after its last
// copy), so what a finished rig held is reused by the next one at once. A stream callback marks the rig done
// when its outputs are in host memory; the worker thread then completes its ticket alone -- a small request
// admitted next to a large one does not wait for the large one.
//
// No kernel here waits on another launch: the aggregation draws its work items from a ticket (every item
// it waits on was drawn earlier), and the pair WTA + median launch only waits on blocks of its own launch, which
// are dispatched as the other rigs' kernels retire. At most kMaxSlots such launches are in flight, so their
// waiting median blocks (8 per launch) never hold every SM.
#include "sister_engine.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>

namespace sister {

namespace {

constexpr size_t kAlign = 256;
constexpr int kMaxSlots = 16;
constexpr size_t kKeepUnwaited = 4096; // finished tickets nobody waited for: the oldest beyond this are dropped
// Rigs of at most this many padded cells (Wp*Hp*dp; 1920x1080 at 256 disparities is 0.99 G) run on high-priority
// streams: when SMs free up, their pending blocks are dispatched before those of larger rigs, so a smaller
// request admitted next to a large one is not held behind every block of the large one.
constexpr double kHighPrioCells = 1.2e9;

size_t al(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

int nmodes_of(const sister_rig &r) { return (r.multi ? 1 : 0) + (r.horiz ? 1 : 0) + (r.vert ? 1 : 0); }

// Buffers of one rig inside its device block, in this order (every offset 256-byte aligned).
struct Layout {
    size_t errflag, rowflags, raw, views, frames, census, wta, med, masks, cost, sum0, sum1, bnd, progress, outs, total;
};
Layout layout(const Geom &g, int channels, int nmodes, const SgmPlan &p) {
    Layout L{};
    const size_t plane = g.plane, vol = plane * g.dp * 2, img = (size_t)g.w * g.h;
    size_t o = 0;
    auto take = [&](size_t n) {
        const size_t at = o;
        o += al(n);
        return at;
    };
    L.errflag = take(sizeof(unsigned));
    L.rowflags = take(4 * (size_t)std::max(g.Wp, g.Hp) * sizeof(unsigned));
    L.raw = take(channels == 3 ? 5 * img * 3 : 0);
    L.views = take(5 * img);
    L.frames = take(8 * plane);
    L.census = take(8 * plane * 8);
    L.wta = take(8 * plane * 2);
    L.med = take(8 * plane * 2);
    L.masks = take(4 * plane);
    L.cost = take(vol);
    L.sum0 = take(sgm_sum_cells(g, true) * 2); // the pass sums of the original image only (no padded map)
    L.sum1 = take(sgm_sum_cells(g, true) * 2);
    L.bnd = take(sgm_bnd_bytes(g, p));
    L.progress = take(sgm_progress_bytes(std::max(p.ngroups, 1)));
    L.outs = take((size_t)nmodes * img * 2);
    L.total = o;
    return L;
}

bool is_pinned(const void *p) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

int validate(const sister_rig &r, std::string *err) {
    char buf[200];
    for (int v = 0; v < 5; v++)
        if (!r.views[v]) {
            std::snprintf(buf, sizeof buf, "view %d is NULL", v);
            *err = buf;
            return SISTER_EINVAL;
        }
    if (r.channels != 1 && r.channels != 3) {
        *err = "channels must be 1 or 3";
        return SISTER_EINVAL;
    }
    if (r.width < 4 || r.height < 4 || (r.width % 4) || (r.height % 4)) {
        std::snprintf(buf, sizeof buf, "size %dx%d: width and height must be positive multiples of 4", r.width,
                      r.height);
        *err = buf;
        return SISTER_EINVAL;
    }
    if (r.stride < r.width * r.channels) {
        *err = "stride < width*channels";
        return SISTER_EINVAL;
    }
    if (r.max_disparity < 8 || r.max_disparity > 512 || (r.max_disparity % 8)) {
        std::snprintf(buf, sizeof buf, "max disparity %d: must be a multiple of 8 in [8, 512]", r.max_disparity);
        *err = buf;
        return SISTER_EINVAL;
    }
    if (!nmodes_of(r)) {
        *err = "no output requested";
        return SISTER_EINVAL;
    }
    return SISTER_OK;
}

} // namespace

struct Engine::Job {
    cudaStream_t st = nullptr; // its slot's stream: high priority for rigs up to kHighPrioCells padded cells
    Engine *eng = nullptr;
    uint64_t ticket = 0;
    sister_rig rig{};
    Geom g{};
    SgmPlan plan{};
    int nmodes = 0;
    size_t bytes = 0;
    int slot = -1;
    char *mem = nullptr;
    bool stage_in = false, stage_out = false;
    unsigned *err_host = nullptr;
    int status = SISTER_EPENDING;
    bool done = false;
    double t_submit = 0, t_end = 0;
    std::string msg;
};

size_t engine_rig_bytes(int w, int h, int dc, int channels, int nmodes, const SgmPlan &plan) {
    return layout(make_geom(w, h, dc), channels, nmodes, plan).total;
}

int Engine::create(Engine **out, int device, size_t budget, const Limits &lim, std::string *err) {
    *out = nullptr;
    Engine *e = new Engine();
    e->device_ = device;
    cudaError_t ce = cudaSetDevice(device);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        *err = "cudaSetDevice failed";
        delete e;
        return SISTER_EDEVICE;
    }
    init_mask_kernels();
    init_sgm_kernels();
    if (!budget) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = fr / 4 * 3;
    }
    e->budget_ = budget;
    e->lim_ = lim;
    e->lim_.max_inflight = std::max(1, std::min(kMaxSlots, lim.max_inflight));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    ce = cudaMemPoolCreate(&e->pool_, &props);
    if (ce == cudaSuccess) {
        // keep freed memory in the pool; reuse it only once its free has completed (never by making one rig's
        // stream wait on another's)
        uint64_t keep = ~0ull;
        int no = 0;
        cudaMemPoolSetAttribute(e->pool_, cudaMemPoolAttrReleaseThreshold, &keep);
        cudaMemPoolSetAttribute(e->pool_, cudaMemPoolReuseAllowInternalDependencies, &no);
    }
    e->streams_.assign(kMaxSlots, nullptr);
    e->streams_hi_.assign(kMaxSlots, nullptr);
    e->pinned_.assign(kMaxSlots, Pinned{});
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    for (int s = 0; s < kMaxSlots && ce == cudaSuccess; s++) {
        ce = cudaStreamCreateWithFlags(&e->streams_[s], cudaStreamNonBlocking);
        if (ce == cudaSuccess)
            ce = cudaStreamCreateWithPriority(&e->streams_hi_[s], cudaStreamNonBlocking, prio_greatest);
        if (ce == cudaSuccess) ce = cudaHostAlloc(&e->pinned_[s].p, kAlign, cudaHostAllocDefault);
        e->pinned_[s].cap = kAlign;
    }
    if (ce != cudaSuccess) {
        cudaGetLastError();
        *err = std::string("engine setup: ") + cudaGetErrorString(ce);
        delete e;
        return ce == cudaErrorMemoryAllocation ? SISTER_ENOMEM : SISTER_EDEVICE;
    }
    for (int s = kMaxSlots - 1; s >= 0; s--) e->free_slots_.push_back(s);
    e->worker_ = std::thread([e] { e->run(); });
    *out = e;
    return SISTER_OK;
}

Engine::~Engine() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    if (worker_.joinable()) worker_.join();
    cudaSetDevice(device_);
    for (auto *v : {&streams_, &streams_hi_})
        for (cudaStream_t s : *v)
            if (s) {
                cudaStreamSynchronize(s);
                cudaStreamDestroy(s);
            }
    for (Pinned &p : pinned_)
        if (p.p) cudaFreeHost(p.p);
    if (pool_) cudaMemPoolDestroy(pool_);
    cudaGetLastError();
    for (auto &kv : jobs_) delete kv.second;
}

const SgmPlan &Engine::plan_for(const Geom &g) {
    std::lock_guard<std::mutex> lk(plan_mu_);
    const uint64_t key = (uint64_t)g.w << 40 | (uint64_t)g.h << 20 | (uint64_t)g.dc;
    auto it = plans_.find(key);
    if (it == plans_.end()) it = plans_.emplace(key, sgm_plan(g, device_)).first;
    return it->second;
}

void Engine::set_limits(const Limits &lim) {
    std::lock_guard<std::mutex> lk(mu_);
    lim_.max_inflight = std::max(1, std::min(kMaxSlots, lim.max_inflight));
    lim_.max_queue = lim.max_queue;
    cv_work_.notify_all();
}

void Engine::stats(uint64_t *admissions, uint64_t *completed, uint64_t *rejected, int *peak_inflight) {
    std::lock_guard<std::mutex> lk(mu_);
    if (admissions) *admissions = admissions_;
    if (completed) *completed = completed_n_;
    if (rejected) *rejected = rejected_;
    if (peak_inflight) *peak_inflight = peak_inflight_;
}

int Engine::submit(const sister_rig &rig, uint64_t *ticket, std::string *err) {
    int rc = validate(rig, err);
    if (rc) return rc;
    cudaSetDevice(device_);
    Job *j = new Job();
    j->eng = this;
    j->rig = rig;
    j->g = make_geom(rig.width, rig.height, rig.max_disparity);
    j->plan = plan_for(j->g);
    if (j->plan.R < 1) {
        delete j;
        *err = "no launch configuration fits the aggregation kernel";
        return SISTER_EDEVICE;
    }
    j->nmodes = nmodes_of(rig);
    j->bytes = layout(j->g, rig.channels, j->nmodes, j->plan).total;
    if (j->bytes > budget_) {
        char buf[200];
        std::snprintf(buf, sizeof buf, "rig %dx%d at max disparity %d needs %zu device bytes; the budget is %zu",
                      rig.width, rig.height, rig.max_disparity, j->bytes, budget_);
        *err = buf;
        delete j;
        return SISTER_EBUDGET;
    }
    std::lock_guard<std::mutex> lk(mu_);
    if (queue_.size() >= lim_.max_queue) {
        rejected_++;
        *err = "request queue full";
        delete j;
        return SISTER_EBUSY;
    }
    j->ticket = next_ticket_++;
    j->t_submit = now_ms();
    jobs_[j->ticket] = j;
    queue_.push_back(j);
    *ticket = j->ticket;
    cv_work_.notify_one();
    return SISTER_OK;
}

int Engine::wait(uint64_t ticket, int timeout_ms, double *latency_ms, std::string *err) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = jobs_.find(ticket);
    if (it == jobs_.end()) {
        *err = "unknown ticket (never issued, already waited for, or dropped unwaited)";
        return SISTER_EINVAL;
    }
    Job *j = it->second;
    if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms), [&] { return j->done; }))
        return SISTER_EPENDING;
    const int st = j->status;
    if (latency_ms) *latency_ms = j->t_end - j->t_submit;
    if (st != SISTER_OK) *err = j->msg;
    jobs_.erase(it);
    delete j;
    return st;
}

bool Engine::can_admit_locked() const {
    return !queue_.empty() && inflight_ < lim_.max_inflight && !free_slots_.empty() &&
           reserved_ + queue_.front()->bytes <= budget_;
}

void CUDART_CB Engine::on_done(void *p) {
    Job *j = static_cast<Job *>(p);
    Engine *e = j->eng;
    {
        std::lock_guard<std::mutex> lk(e->mu_);
        e->completed_.push_back(j);
    }
    e->cv_work_.notify_one();
}

void Engine::run() {
    cudaSetDevice(device_);
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
        cv_work_.wait(lk, [&] { return !completed_.empty() || can_admit_locked() || (stop_ && queue_.empty() && !inflight_); });
        while (!completed_.empty()) {
            Job *j = completed_.back();
            completed_.pop_back();
            lk.unlock();
            finish(j);
            lk.lock();
        }
        while (can_admit_locked()) {
            Job *j = queue_.front();
            queue_.pop_front();
            j->slot = free_slots_.back();
            free_slots_.pop_back();
            j->st = (double)j->g.plane * j->g.dp <= kHighPrioCells ? streams_hi_[j->slot] : streams_[j->slot];
            reserved_ += j->bytes;
            inflight_++;
            peak_inflight_ = std::max(peak_inflight_, inflight_);
            admissions_++;
            lk.unlock();
            admit(j);
            lk.lock();
        }
        if (stop_ && queue_.empty() && !inflight_ && completed_.empty()) return;
    }
}

void Engine::admit(Job *j) {
    const sister_rig &r = j->rig;
    const int w = r.width, h = r.height, ch = r.channels;
    const size_t img = (size_t)w * h, in_bytes = 5 * img * ch, out_bytes = (size_t)j->nmodes * img * 2;
    j->stage_in = false;
    for (int v = 0; v < 5; v++) j->stage_in = j->stage_in || !is_pinned(r.views[v]);
    j->stage_out = false;
    for (uint16_t *o : {r.multi, r.horiz, r.vert})
        if (o) j->stage_out = j->stage_out || !is_pinned(o);
    // per-slot pinned staging: the error flag, then staged inputs, then staged outputs (grown when needed; the
    // slot's previous rig has completed, so its staging is idle)
    Pinned &pin = pinned_[j->slot];
    const size_t need = kAlign + (j->stage_in ? al(in_bytes) : 0) + (j->stage_out ? al(out_bytes) : 0);
    std::string err;
    int status = SISTER_OK;
    if (pin.cap < need) {
        cudaFreeHost(pin.p);
        pin.p = nullptr;
        pin.cap = 0;
        if (cudaHostAlloc(&pin.p, need, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            pin.p = nullptr;
            status = SISTER_ENOMEM;
            err = "pinned staging allocation failed";
        } else {
            pin.cap = need;
        }
    }
    if (status == SISTER_OK) {
        j->err_host = static_cast<unsigned *>(pin.p);
        *j->err_host = kErrNone;
        if (j->stage_in) {
            uint8_t *dst = static_cast<uint8_t *>(pin.p) + kAlign;
            const size_t row = (size_t)w * ch;
            for (int v = 0; v < 5; v++)
                for (int y = 0; y < h; y++)
                    std::memcpy(dst + (size_t)v * row * h + (size_t)y * row, r.views[v] + (size_t)y * r.stride, row);
        }
        status = enqueue(j, &err);
    }
    if (status != SISTER_OK) {
        // nothing of this rig remains queued on its stream once it is synchronised
        cudaStream_t st = j->st;
        cudaStreamSynchronize(st);
        if (j->mem) cudaFreeAsync(j->mem, st);
        cudaStreamSynchronize(st);
        cudaGetLastError();
        j->mem = nullptr;
        j->status = status;
        j->msg = err;
        std::lock_guard<std::mutex> lk(mu_);
        completed_.push_back(j);
    }
}

int Engine::enqueue(Job *j, std::string *err) {
    const sister_rig &r = j->rig;
    const Geom &g = j->g;
    const int w = r.width, h = r.height, ch = r.channels;
    const size_t img = (size_t)w * h;
    cudaStream_t st = j->st;
    const Layout L = layout(g, ch, j->nmodes, j->plan);
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void **>(&j->mem), L.total, pool_, st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        j->mem = nullptr;
        *err = std::string("device allocation: ") + cudaGetErrorString(e);
        return SISTER_ENOMEM;
    }
    char *b = j->mem;
    unsigned *errflag = reinterpret_cast<unsigned *>(b + L.errflag);
    unsigned *rowflags = reinterpret_cast<unsigned *>(b + L.rowflags);
    uint8_t *views = reinterpret_cast<uint8_t *>(b + L.views);
    uint64_t *census = reinterpret_cast<uint64_t *>(b + L.census);
    uint16_t *wta = reinterpret_cast<uint16_t *>(b + L.wta), *med = reinterpret_cast<uint16_t *>(b + L.med);
    uint8_t *masks = reinterpret_cast<uint8_t *>(b + L.masks);
    // a fresh block holds anything: the error flag and the row flags (epoch 1 marks a published row) start at 0
    e = cudaMemsetAsync(errflag, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(rowflags, 0, 4 * (size_t)std::max(g.Wp, g.Hp) * sizeof(unsigned), st);
    const size_t row = (size_t)w * ch;
    const uint8_t *src[5];
    uint8_t *dst = ch == 3 ? reinterpret_cast<uint8_t *>(b + L.raw) : views;
    for (int v = 0; v < 5 && e == cudaSuccess; v++) {
        const uint8_t *s = j->stage_in ? static_cast<uint8_t *>(pinned_[j->slot].p) + kAlign + (size_t)v * row * h
                                       : r.views[v];
        const size_t spitch = j->stage_in ? row : (size_t)r.stride;
        e = cudaMemcpy2DAsync(dst + (size_t)v * row * h, row, s, spitch, row, h, cudaMemcpyHostToDevice, st);
        src[v] = dst + (size_t)v * row * h;
    }
    if (e != cudaSuccess) {
        *err = std::string("uploading views: ") + cudaGetErrorString(e);
        return SISTER_EDEVICE;
    }
    if (ch == 3) launch_to_gray(src, (int)row, 3, w, h, views, st);
    launch_frames(views, g, reinterpret_cast<uint8_t *>(b + L.frames), st);
    launch_census(reinterpret_cast<uint8_t *>(b + L.frames), g, census, st);
    launch_wta_median(census, g, wta, med, rowflags, 1u, errflag, st);
    launch_lrc_mask(med, g, masks, st);
    uint16_t *outs[3] = {r.multi, r.horiz, r.vert};
    int k = 0;
    for (int mode = 0; mode < 3; mode++) {
        if (!outs[mode]) continue;
        uint16_t *dout = reinterpret_cast<uint16_t *>(b + L.outs) + (size_t)k * img;
        uint16_t *cost = reinterpret_cast<uint16_t *>(b + L.cost);
        launch_masked_cost(census, masks, g, mode, cost, st);
        SgmRig a{};
        a.cost = cost;
        a.sum0 = reinterpret_cast<uint16_t *>(b + L.sum0);
        a.sum1 = reinterpret_cast<uint16_t *>(b + L.sum1);
        a.bnd = reinterpret_cast<uint16_t *>(b + L.bnd);
        a.progress = reinterpret_cast<unsigned *>(b + L.progress);
        sgm_crop_window(a, g);
        a.out = dout; // the final WTA runs in the aggregation launch
        e = launch_sgm(g, j->plan, a, errflag, st, wait_limit_us_);
        uint16_t *hdst = j->stage_out ? reinterpret_cast<uint16_t *>(static_cast<char *>(pinned_[j->slot].p) + kAlign +
                                                                     (j->stage_in ? al(5 * img * ch) : 0)) +
                                            (size_t)k * img
                                      : outs[mode];
        if (e == cudaSuccess) e = cudaMemcpyAsync(hdst, dout, img * 2, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) {
            *err = std::string("aggregation / output: ") + cudaGetErrorString(e);
            return SISTER_EDEVICE;
        }
        k++;
    }
    e = cudaMemcpyAsync(j->err_host, errflag, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaFreeAsync(j->mem, st);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(st, &Engine::on_done, j);
    if (e != cudaSuccess) {
        *err = std::string("enqueue: ") + cudaGetErrorString(e);
        return SISTER_EDEVICE;
    }
    j->mem = nullptr; // freed in stream order
    return SISTER_OK;
}

void Engine::finish(Job *j) {
    if (j->status == SISTER_EPENDING) { // ran on the device
        j->status = SISTER_OK;
        const unsigned flag = *j->err_host;
        if (flag != kErrNone) {
            j->status = SISTER_ETIMEOUT;
            j->msg = "a bounded device-side wait expired (device reported timeout)";
        } else if (j->stage_out) {
            const sister_rig &r = j->rig;
            const size_t img = (size_t)r.width * r.height;
            const uint16_t *src = reinterpret_cast<const uint16_t *>(
                static_cast<char *>(pinned_[j->slot].p) + kAlign + (j->stage_in ? al(5 * img * r.channels) : 0));
            int k = 0;
            for (uint16_t *o : {r.multi, r.horiz, r.vert})
                if (o) std::memcpy(o, src + (size_t)(k++) * img, img * 2);
        }
    }
    std::lock_guard<std::mutex> lk(mu_);
    reserved_ -= j->bytes;
    inflight_--;
    free_slots_.push_back(j->slot);
    j->t_end = now_ms();
    j->done = true;
    completed_n_++;
    unwaited_.push_back(j->ticket);
    while (unwaited_.size() > kKeepUnwaited) {
        auto it = jobs_.find(unwaited_.front());
        unwaited_.pop_front();
        if (it != jobs_.end() && it->second->done) {
            delete it->second;
            jobs_.erase(it);
        }
    }
    cv_done_.notify_all();
}

} // namespace sister
