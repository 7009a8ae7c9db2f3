// Allocation-free aggregation entry point.
//
// Some callers cannot allocate device memory at the time they need a result: a robot's perception
// loop or a ROS service callback with a fixed, pre-reserved memory budget and hard latency limits,
// code running inside another framework that owns every device allocation, or a process that must not
// touch the CUDA allocator after start-up. sister_aggregate_static serves them: it runs the 8-path
// aggregation + winner-take-all of sister_compute on a cost volume the caller already holds, and keeps
// all of its scratch (the two pass sums, hand-off records, progress counters, error flag) in one file-scope
// device array of fixed size instead of calling cudaMalloc.
#include "sister_gb300.h"
#include "sister_internal.h"

#include <cstdio>
#include <cstring>
#include <mutex>

using namespace sister;

namespace {

// Scratch arena: loaded with the library's device code and held by every GPU that loads it, until exit.
constexpr size_t kStaticScratchBytes = (size_t)SISTER_STATIC_SCRATCH_BYTES;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {};

int report(char *err, size_t errlen, int code, const char *msg) {
    if (err && errlen) {
        std::snprintf(err, errlen, "%s", msg);
    }
    return code;
}

// Device address of the arena for the current device; looked up once per device with that device
// current (the host-side symbol is only a stand-in and must never be passed to a kernel).
int scratch_for_device(int dev, void **out, char *err, size_t errlen) {
    if (dev < 0 || dev >= kMaxDevices) return report(err, errlen, SISTER_EDEVICE, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            char buf[256];
            std::snprintf(buf, sizeof buf, "cudaGetSymbolAddress of the scratch arena failed: %s", cudaGetErrorString(e));
            return report(err, errlen, SISTER_EDEVICE, buf);
        }
        init_sgm_kernels(); // dynamic shared-memory limits of the aggregation kernels on this device
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return SISTER_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

} // namespace

extern "C" int sister_aggregate_static(const uint16_t *cost, int width, int height, int dc, int dstride,
                                       uint16_t *out, uint16_t *disp_padded, void *stream, char *err,
                                       size_t errlen) {
    if (err && errlen) err[0] = 0;
    if (!cost) return report(err, errlen, SISTER_EINVAL, "cost volume pointer is NULL");
    if (reinterpret_cast<uintptr_t>(cost) & 15)
        return report(err, errlen, SISTER_EINVAL, "cost volume pointer must be 16-byte aligned");
    if (width < 4 || height < 4 || (width % 4) || (height % 4))
        return report(err, errlen, SISTER_EINVAL, "width and height must be positive multiples of 4");
    if (dc < 8 || dc > 512 || (dc % 8))
        return report(err, errlen, SISTER_EINVAL, "max disparity must be a multiple of 8 in [8, 512]");
    const Geom g = make_geom(width, height, dc);
    if (dstride != g.dp) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "cost d-stride %d does not match the layout for max disparity %d (expected %d)",
                      dstride, dc, g.dp);
        return report(err, errlen, SISTER_EINVAL, buf);
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return report(err, errlen, SISTER_EDEVICE, "no current CUDA device");
    }
    void *base = nullptr;
    int rc = scratch_for_device(dev, &base, err, errlen);
    if (rc) return rc;

    // tallest bands: the fewest hand-off records for the arena (the arena, not parallelism, is the constraint)
    const SgmPlan p = sgm_plan(g, dev, 64);
    if (p.R < 1) return report(err, errlen, SISTER_EDEVICE, "no launch configuration fits the aggregation kernel");
    const size_t sum_bytes = align256(g.plane * g.dp * sizeof(uint16_t));
    const size_t bnd_bytes = align256(sgm_bnd_bytes(g, p));
    const size_t prog_bytes = align256(sgm_progress_bytes(p.ngroups));
    const size_t need = 2 * sum_bytes + bnd_bytes + prog_bytes + 256;
    if (need > kStaticScratchBytes) {
        char buf[256];
        std::snprintf(buf, sizeof buf,
                      "rig %dx%d at max disparity %d needs %zu bytes of scratch; the static arena holds %zu",
                      width, height, dc, need, kStaticScratchBytes);
        return report(err, errlen, SISTER_EBUDGET, buf);
    }
    unsigned char *b = static_cast<unsigned char *>(base);
    SgmRig a{};
    a.cost = cost;
    a.sum0 = reinterpret_cast<uint16_t *>(b);
    a.sum1 = reinterpret_cast<uint16_t *>(b + sum_bytes);
    a.bnd = reinterpret_cast<uint16_t *>(b + 2 * sum_bytes);
    a.progress = reinterpret_cast<unsigned *>(b + 2 * sum_bytes + bnd_bytes);
    unsigned *errflag = reinterpret_cast<unsigned *>(b + 2 * sum_bytes + bnd_bytes + prog_bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the arena keeps the previous call's contents: the error flag must start at zero (the progress
    // counters are cleared by the aggregation launch)
    cudaError_t e = cudaMemsetAsync(errflag, 0, sizeof(unsigned), st);
    if (e == cudaSuccess) e = launch_sgm(g, p, a, errflag, st);
    if (e == cudaSuccess) e = launch_sgm_wta(g, a.sum0, a.sum1, out, disp_padded, st, false); // whole-plane sums
    unsigned flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, errflag, sizeof flag, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[200];
        std::snprintf(buf, sizeof buf, "aggregation failed: %s", cudaGetErrorString(e));
        return report(err, errlen, SISTER_EDEVICE, buf);
    }
    if (flag != kErrNone) return report(err, errlen, SISTER_ETIMEOUT, "a bounded device-side wait expired");
    return SISTER_OK;
}
