// Batched execution of many rigs (sister_batch_*): the throughput path for callers with many independent
// rigs at once, e.g. the 64 mixed-size rigs of one batch.
//
// One call computes every rig exactly as sister_compute would (same kernels, bit-identical outputs), through
// the request engine (sister_engine.cu): the rigs are admitted one after another as stream slots and device
// memory free up -- a rig starts while earlier ones are still on the GPU, so the stages of several rigs overlap,
// and the memory of a finished rig is reused at once -- and the call returns when the last one has landed.
#include "sister_engine.h"

#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

using namespace sister;

struct sister_batch {
    Engine *eng = nullptr;
    std::string err;
};

extern "C" {

size_t sister_batch_rig_bytes(int width, int height, int max_disparity, int nmodes) {
    if (width < 4 || height < 4 || max_disparity < 8 || max_disparity > 512 || nmodes < 0) return 0;
    const Geom g = make_geom(width, height, max_disparity);
    if (g.dpl < 0) return 0;
    int dev = 0;
    SgmPlan p{};
    if (cudaGetDevice(&dev) == cudaSuccess) {
        init_sgm_kernels();
        p = sgm_plan(g, dev);
    }
    cudaGetLastError();
    if (p.R < 1) p = sgm_plan_gb300(g);
    if (p.R < 1) return 0;
    return engine_rig_bytes(width, height, max_disparity, 3, nmodes, p);
}

int sister_batch_create(sister_batch **out, int device, size_t budget_bytes) {
    if (!out) return SISTER_EINVAL;
    *out = nullptr;
    sister_batch *b = new sister_batch();
    Engine::Limits lim;
    lim.max_queue = (size_t)-1; // a batch queues all of its rigs at once
    std::string err;
    const int rc = Engine::create(&b->eng, device, budget_bytes, lim, &err);
    if (rc != SISTER_OK) {
        delete b;
        return rc;
    }
    *out = b;
    return SISTER_OK;
}

void sister_batch_destroy(sister_batch *b) {
    if (!b) return;
    delete b->eng;
    delete b;
}

const char *sister_batch_last_error(sister_batch *b) { return b ? b->err.c_str() : "null batch"; }

int sister_batch_run(sister_batch *b, const sister_rig *rigs, int nrigs) {
    if (!b) return SISTER_EINVAL;
    if (nrigs < 0 || (nrigs > 0 && !rigs)) {
        b->err = "rigs is NULL";
        return SISTER_EINVAL;
    }
    // every rig is checked before any runs: a bad rig or one that alone exceeds the budget fails the call
    for (int k = 0; k < nrigs; k++) {
        const sister_rig &r = rigs[k];
        const int nm = (r.multi ? 1 : 0) + (r.horiz ? 1 : 0) + (r.vert ? 1 : 0);
        char buf[320];
        if (!nm) continue;
        bool ok = r.width >= 4 && r.height >= 4 && !(r.width % 4) && !(r.height % 4) && r.max_disparity >= 8 &&
                  r.max_disparity <= 512 && !(r.max_disparity % 8) && (r.channels == 1 || r.channels == 3) &&
                  r.stride >= r.width * r.channels;
        for (int v = 0; v < 5; v++) ok = ok && r.views[v];
        if (!ok) {
            std::snprintf(buf, sizeof buf,
                          "rig %d: %dx%d, %d channels, stride %d, max disparity %d: sizes must be positive multiples "
                          "of 4, channels 1 or 3, stride >= width*channels, max disparity a multiple of 8 in "
                          "[8, 512], views non-NULL",
                          k, r.width, r.height, r.channels, r.stride, r.max_disparity);
            b->err = buf;
            return SISTER_EINVAL;
        }
        const Geom g = make_geom(r.width, r.height, r.max_disparity);
        const size_t need = engine_rig_bytes(r.width, r.height, r.max_disparity, r.channels, nm,
                                             sgm_plan(g, b->eng->device()));
        if (need > b->eng->budget()) {
            std::snprintf(buf, sizeof buf, "rig %d (%dx%d, max disparity %d) needs %zu bytes; the batch budget is %zu",
                          k, r.width, r.height, r.max_disparity, need, b->eng->budget());
            b->err = buf;
            return SISTER_EBUDGET;
        }
    }
    std::vector<uint64_t> tickets;
    tickets.reserve(nrigs);
    int rc = SISTER_OK;
    std::string err;
    for (int k = 0; k < nrigs; k++) {
        const sister_rig &r = rigs[k];
        if (!r.multi && !r.horiz && !r.vert) continue;
        uint64_t t = 0;
        const int s = b->eng->submit(r, &t, &err);
        if (s != SISTER_OK) {
            rc = s;
            b->err = err;
            break;
        }
        tickets.push_back(t);
    }
    // every submitted rig is waited for (its buffers are the caller's), the first failure is reported
    for (uint64_t t : tickets) {
        std::string e2;
        const int s = b->eng->wait(t, 1 << 30, nullptr, &e2);
        if (s != SISTER_OK && rc == SISTER_OK) {
            rc = s;
            b->err = e2;
        }
    }
    return rc;
}

} // extern "C"
