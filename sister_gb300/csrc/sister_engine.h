// Request engine of the serving loop (sister_server_*): continuous
// admission of independent rigs against a device-memory budget, each admitted rig computed on its own stream.
#pragma once

#include "sister_gb300.h"
#include "sister_internal.h"

#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace sister {

// Device bytes one admitted rig holds while it is computed: the stages before the aggregation, one set of
// aggregation volumes (the requested modes run one after another on the rig's stream and share them) and the
// output image of every requested mode.
size_t engine_rig_bytes(int w, int h, int dc, int channels, int nmodes, const SgmPlan &plan);

class Engine {
  public:
    struct Limits {
        int max_inflight = 8;  // rigs computed at once (one stream each)
        size_t max_queue = 1024; // requests waiting for admission; beyond it submit returns SISTER_EBUSY
    };
    // budget: device bytes the admitted rigs may hold together (0: three quarters of the free memory)
    static int create(Engine **out, int device, size_t budget, const Limits &lim, std::string *err);
    ~Engine(); // finishes every admitted and queued request first

    // Validates the rig and queues it. SISTER_EINVAL (bad rig), SISTER_EBUDGET (the rig alone exceeds the
    // budget), SISTER_EBUSY (queue full); nothing is queued then.
    int submit(const sister_rig &rig, uint64_t *ticket, std::string *err);
    // The request's status once its outputs are in host memory (the ticket is then released), or SISTER_EPENDING
    // when it is still queued or running after timeout_ms (the ticket stays valid). latency: submit -> outputs.
    int wait(uint64_t ticket, int timeout_ms, double *latency_ms, std::string *err);
    void set_limits(const Limits &lim);
    void stats(uint64_t *admissions, uint64_t *completed, uint64_t *rejected, int *peak_inflight);
    size_t budget() const { return budget_; }
    int device() const { return device_; }
    void set_wait_limit_us(unsigned us) { wait_limit_us_ = us; }

    struct Job;

  private:
    Engine() = default;
    void run();
    bool can_admit_locked() const;
    void admit(Job *j);                       // called without the lock held
    void finish(Job *j);                      // called without the lock held
    int enqueue(Job *j, std::string *err);    // the rig's pipeline on its stream
    const SgmPlan &plan_for(const Geom &g);   // cached per geometry
    static void CUDART_CB on_done(void *job); // stream callback: the rig's outputs have landed

    int device_ = 0;
    size_t budget_ = 0, reserved_ = 0;
    Limits lim_;
    unsigned wait_limit_us_ = kDefaultWaitUs;
    cudaMemPool_t pool_ = nullptr;
    std::vector<cudaStream_t> streams_;    // per slot, default priority
    std::vector<cudaStream_t> streams_hi_; // per slot, the device's highest priority (smaller rigs)
    std::vector<int> free_slots_;
    struct Pinned {
        void *p = nullptr;
        size_t cap = 0;
    };
    std::vector<Pinned> pinned_; // per slot: staging of pageable inputs / outputs and the error flag

    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<Job *> queue_;
    std::vector<Job *> completed_;
    std::unordered_map<uint64_t, Job *> jobs_;
    std::deque<uint64_t> unwaited_; // finished tickets in completion order (bounded; oldest evicted)
    std::map<uint64_t, SgmPlan> plans_;
    std::mutex plan_mu_;
    uint64_t next_ticket_ = 1;
    int inflight_ = 0, peak_inflight_ = 0;
    uint64_t admissions_ = 0, completed_n_ = 0, rejected_ = 0;
    bool stop_ = false;
    std::thread worker_;
};

} // namespace sister
