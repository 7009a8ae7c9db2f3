// Serving loop (sister_server_*): requests (one rig each, the shape of the reference's ROS service request,
// ros/README.md:6-15: dispCount + five images -> disparity images) are submitted from any host thread and
// computed by the request engine (sister_engine.cu) with continuous admission: a request starts as soon as a
// stream slot is free and its device memory fits the budget beside the requests already running, overlaps with
// them on the device, and its ticket completes when its own outputs are in host memory.
#include "sister_engine.h"

#include <mutex>
#include <string>

using namespace sister;

struct sister_server {
    Engine *eng = nullptr;
    std::mutex mu;
    std::string err;
    void set_err(const std::string &e) {
        std::lock_guard<std::mutex> lk(mu);
        err = e;
    }
};

extern "C" {

int sister_server_create(sister_server **out, int device, size_t budget_bytes) {
    if (!out) return SISTER_EINVAL;
    *out = nullptr;
    sister_server *s = new sister_server();
    std::string err;
    int rc = Engine::create(&s->eng, device, budget_bytes, Engine::Limits{}, &err);
    if (rc != SISTER_OK) {
        delete s;
        return rc;
    }
    *out = s;
    return SISTER_OK;
}

void sister_server_destroy(sister_server *s) {
    if (!s) return;
    delete s->eng;
    delete s;
}

const char *sister_server_last_error(sister_server *s) {
    // a copy owned by the calling thread: valid until this thread's next call
    static thread_local std::string copy;
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    copy = s->err;
    return copy.c_str();
}

int sister_server_set_limits(sister_server *s, int max_inflight, size_t max_queue) {
    if (!s || max_inflight < 1) return SISTER_EINVAL;
    Engine::Limits lim;
    lim.max_inflight = max_inflight;
    lim.max_queue = max_queue;
    s->eng->set_limits(lim);
    return SISTER_OK;
}

int sister_server_submit(sister_server *s, const sister_rig *rig, uint64_t *ticket) {
    if (!s || !rig || !ticket) return SISTER_EINVAL;
    std::string err;
    const int rc = s->eng->submit(*rig, ticket, &err);
    if (rc != SISTER_OK) s->set_err(err);
    return rc;
}

int sister_server_wait(sister_server *s, uint64_t ticket, int timeout_ms, double *latency_ms) {
    if (!s) return SISTER_EINVAL;
    std::string err;
    const int rc = s->eng->wait(ticket, timeout_ms, latency_ms, &err);
    if (rc != SISTER_OK && rc != SISTER_EPENDING) s->set_err(err);
    return rc;
}

int sister_server_stats(sister_server *s, uint64_t *admitted, uint64_t *completed, uint64_t *rejected,
                        int *peak_inflight) {
    if (!s) return SISTER_EINVAL;
    s->eng->stats(admitted, completed, rejected, peak_inflight);
    return SISTER_OK;
}

} // extern "C"
