// Serving loop (sister_server_*): requests (one rig each, the shape of the reference's ROS service
// request, ros/README.md:6-15: dispCount + five images -> disparity images) arrive on any host thread; a
// worker thread keeps the GPU busy by draining the queue into dynamic batches whose device memory fits the
// server's budget (the batch engine of sister_batch.cu), in arrival order, and completes each request's
// ticket when its outputs are in host memory. A request admitted into a batch waits for that batch only;
// requests arriving meanwhile form the next batch as soon as the engine is free.
#include "sister_gb300.h"
#include "sister_internal.h"

#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace {

struct Req {
    uint64_t ticket;
    sister_rig rig;
    size_t bytes;
};

struct Done {
    int status = 1; // 1: pending
    double submit_ms = 0, start_ms = 0, end_ms = 0;
};

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

} // namespace

struct sister_server {
    sister_batch *batch = nullptr;
    size_t budget = 0;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;
    std::unordered_map<uint64_t, Done> done;
    uint64_t next_ticket = 1;
    bool stop = false;
    size_t max_batch = 64;
    std::string err;
    uint64_t batches = 0, rigs = 0;

    void run() {
        std::vector<Req> take;
        std::vector<sister_rig> rigs_v;
        for (;;) {
            take.clear();
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait(lk, [&] { return stop || !queue.empty(); });
                if (stop && queue.empty()) return;
                // dynamic batch: queued requests in arrival order while they fit the budget (the first always)
                size_t used = 0;
                while (!queue.empty() && take.size() < max_batch &&
                       (take.empty() || used + queue.front().bytes <= budget)) {
                    used += queue.front().bytes;
                    take.push_back(queue.front());
                    queue.pop_front();
                }
                const double t = now_ms();
                for (const Req &r : take) done[r.ticket].start_ms = t;
            }
            rigs_v.clear();
            for (const Req &r : take) rigs_v.push_back(r.rig);
            int rc = sister_batch_run(batch, rigs_v.data(), (int)rigs_v.size());
            if (rc != SISTER_OK && take.size() > 1) {
                // one bad request must not fail the others: run them one by one to attribute the status
                for (size_t q = 0; q < take.size(); q++) {
                    const int rq = sister_batch_run(batch, &rigs_v[q], 1);
                    std::lock_guard<std::mutex> lk(mu);
                    Done &d = done[take[q].ticket];
                    d.status = rq;
                    d.end_ms = now_ms();
                    if (rq != SISTER_OK) err = sister_batch_last_error(batch);
                }
            } else {
                std::lock_guard<std::mutex> lk(mu);
                const double t = now_ms();
                for (const Req &r : take) {
                    Done &d = done[r.ticket];
                    d.status = rc;
                    d.end_ms = t;
                }
                if (rc != SISTER_OK) err = sister_batch_last_error(batch);
            }
            {
                std::lock_guard<std::mutex> lk(mu);
                batches++;
                rigs += take.size();
            }
            cv_done.notify_all();
        }
    }
};

extern "C" {

int sister_server_create(sister_server **out, int device, size_t budget_bytes) {
    if (!out) return SISTER_EINVAL;
    *out = nullptr;
    sister_server *s = new sister_server();
    int rc = sister_batch_create(&s->batch, device, budget_bytes);
    if (rc != SISTER_OK) {
        delete s;
        return rc;
    }
    // the engine reserves staging room inside the arena; requests are admitted against what remains
    if (!budget_bytes) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget_bytes = fr;
    }
    s->budget = budget_bytes > (16u << 20) ? budget_bytes - (16u << 20) : 0;
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return SISTER_OK;
}

void sister_server_destroy(sister_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    sister_batch_destroy(s->batch);
    delete s;
}

const char *sister_server_last_error(sister_server *s) { return s ? s->err.c_str() : "null server"; }

int sister_server_submit(sister_server *s, const sister_rig *rig, uint64_t *ticket) {
    if (!s || !rig || !ticket) return SISTER_EINVAL;
    const int nmodes = (rig->multi ? 1 : 0) + (rig->horiz ? 1 : 0) + (rig->vert ? 1 : 0);
    const size_t bytes = sister_batch_rig_bytes(rig->width, rig->height, rig->max_disparity, nmodes);
    if (!bytes) return SISTER_EINVAL;
    if (bytes > s->budget) return SISTER_EBUDGET;
    std::lock_guard<std::mutex> lk(s->mu);
    Req r{s->next_ticket++, *rig, bytes};
    s->done[r.ticket].submit_ms = now_ms();
    s->queue.push_back(r);
    *ticket = r.ticket;
    s->cv_work.notify_one();
    return SISTER_OK;
}

int sister_server_wait(sister_server *s, uint64_t ticket, int timeout_ms, double *latency_ms) {
    if (!s) return SISTER_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->done.find(ticket);
    if (it == s->done.end()) return SISTER_EINVAL;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                        [&] { return s->done[ticket].status != 1; });
    if (!ok) return SISTER_ETIMEOUT;
    const Done d = s->done[ticket];
    s->done.erase(ticket);
    if (latency_ms) *latency_ms = d.end_ms - d.submit_ms;
    return d.status;
}

int sister_server_stats(sister_server *s, uint64_t *batches, uint64_t *rigs) {
    if (!s) return SISTER_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    if (batches) *batches = s->batches;
    if (rigs) *rigs = s->rigs;
    return SISTER_OK;
}

} // extern "C"
