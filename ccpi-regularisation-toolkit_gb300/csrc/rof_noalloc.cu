// ROF-TV entry point that performs no device memory allocation.
//
// Who needs it: callers that cannot call cudaMalloc (or any allocator) at the
// moment they regularise — typically a reconstruction or learning framework
// that has already claimed the GPU's memory for its own caching allocator or
// fixed memory budget, so a fresh allocation would fail or break its
// accounting, and real-time pipelines that forbid allocation (which can
// synchronise the device and can fail under memory pressure) after start-up.
//
// How: the only scratch the ROF iteration needs beyond the caller's input and
// output — the second ping-pong copy of U, the FP64 reduction slots of the
// stopping rule and the stop-control block — lives in one file-scope device
// array, g_rof_noalloc_scratch, of fixed size (68 MiB + 256 B).  Every GPU on
// which this module is loaded holds that array until the process exits.
//
// Limits and rules for callers:
//   * at most kNoAllocMaxVoxels = 2^24 voxels (e.g. 256^3 or 4096^2); larger
//     inputs are rejected with status -2 and a message;
//   * with epsil != 0 the shape must need at most 2^18 reduction blocks;
//   * every call uses the same array, which keeps the last call's contents:
//     calls whose GPU work overlaps (two streams, or two host threads) race
//     on it and must be serialised by the caller;
//   * the first call on each device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current);
//   * a call waits for its stream before it returns (it reads the stop
//     control back), so it cannot be captured into a CUDA graph; with
//     epsil != 0 it also reads the stop flag every twentieth iteration and
//     stops enqueueing once the rule has fired.
#include <mutex>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"

namespace cilreg {
namespace {

constexpr long long kNoAllocMaxVoxels = 1LL << 24;
constexpr long long kNoAllocMaxPartials = 1LL << 18;
constexpr size_t kUBytes = (size_t)kNoAllocMaxVoxels * sizeof(float);        // 64 MiB
constexpr size_t kPartBytes = (size_t)kNoAllocMaxPartials * sizeof(double2);  // 4 MiB
constexpr size_t kCtlBytes = 256;
constexpr size_t kScratchBytes = kUBytes + kPartBytes + kCtlBytes;

// The whole scratch of cilreg_rof_tv_dev_noalloc.  In host code this name is
// only a host-side stand-in: the device address comes from
// cudaGetSymbolAddress below and is what the kernels receive.
static __device__ __align__(256) unsigned char g_rof_noalloc_scratch[kScratchBytes];

struct DeviceScratch {
    std::mutex lock;
    unsigned char* ptr = nullptr;
};
DeviceScratch g_scratch_of_device[64];

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
int scratch_on_current_device(unsigned char** out) {
    int dev = -1;
    CILREG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return fail(ERR_ARG, __FILE__, __LINE__, "device index %d not supported", dev);
    DeviceScratch& s = g_scratch_of_device[dev];
    std::lock_guard<std::mutex> guard(s.lock);
    if (!s.ptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_rof_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(ERR_CUDA, __FILE__, __LINE__, "cudaGetSymbolAddress of the no-allocation scratch failed: %s",
                        cudaGetErrorString(e));
        s.ptr = (unsigned char*)p;
    }
    *out = s.ptr;
    return OK;
}

}  // namespace
}  // namespace cilreg

using namespace cilreg;

extern "C" int cilreg_rof_tv_dev_noalloc(const float* d_in, float* d_out, float* infovector, const float* d_lambda,
                                         float lambdaPar, int iters, float tau, float epsil, int dimX, int dimY,
                                         int dimZ, void* stream) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    if (!d_in || !d_out) return fail(ERR_ARG, __FILE__, __LINE__, "null device pointer");
    if (d_in == d_out) return fail(ERR_ARG, __FILE__, __LINE__, "input and output must be distinct buffers");
    const Dims d = make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ);
    if (d.n > kNoAllocMaxVoxels)
        return fail(ERR_ARG, __FILE__, __LINE__,
                    "%lld voxels exceed the no-allocation limit of %lld voxels (use cilreg_rof_tv_dev)", d.n,
                    kNoAllocMaxVoxels);
    CILREG_TRY(rof_check_grid(d));  // the same limit as cilreg_rof_tv_dev, from the plan that runs
    const long long nparts = rof_partial_slots(d);
    if (epsil != 0.0f && nparts > kNoAllocMaxPartials)
        return fail(ERR_ARG, __FILE__, __LINE__,
                    "shape (%d, %d, %d) needs %lld reduction slots; the no-allocation limit is %lld", dimX, dimY,
                    dimZ, nparts, kNoAllocMaxPartials);

    unsigned char* base = nullptr;
    CILREG_TRY(scratch_on_current_device(&base));
    float* alt = (float*)base;
    double2* partials = (double2*)(base + kUBytes);
    StopCtl* ctl = (StopCtl*)(base + kUBytes + kPartBytes);
    cudaStream_t s = (cudaStream_t)stream;

    // the array keeps the previous call's state: reset the stop control; the
    // U buffer and the partials are fully written before they are read
    CILREG_TRY(launch_init_ctl(ctl, iters, s));
    CILREG_CUDA(cudaMemcpyAsync(d_out, d_in, sizeof(float) * (size_t)d.n, cudaMemcpyDeviceToDevice, s));
    float* bufs[2] = {d_out, alt};
    for (int it = 0; it < iters; it++) {
        const int check = (epsil != 0.0f && (it % 5) == 0) ? 1 : 0;
        CILREG_TRY(rof_launch_step(bufs[it & 1], bufs[(it + 1) & 1], d_in, d_lambda, lambdaPar, tau, d, ctl, check,
                                   partials, s));
        if (check) {
            CILREG_TRY(launch_finalize_check(partials, nparts, ctl, epsil, it, s));
            // every fourth check, read the stop flag (a copy into host stack
            // memory, no allocation) and stop enqueueing iterations that
            // would only return at once
            if ((it / 5) % 4 == 3) {
                int stop = 0;
                CILREG_CUDA(cudaMemcpyAsync(&stop, &ctl->stop, sizeof(int), cudaMemcpyDeviceToHost, s));
                CILREG_CUDA(cudaStreamSynchronize(s));
                if (stop) break;
            }
        }
    }
    if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl, iters, bufs, d_out, d.n, s));
    StopCtl h;
    CILREG_CUDA(cudaMemcpyAsync(&h, ctl, sizeof(StopCtl), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (infovector) {
        infovector[0] = (float)h.iters;
        infovector[1] = h.re;
    }
    return OK;
}
