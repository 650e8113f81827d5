// Host runtime shared by all regulariser drivers: error reporting, per-thread
// streams, stream-ordered scratch allocation and the device-side stopping
// control.  Nothing here synchronises the device per iteration.
#pragma once

#include <stdlib.h>

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "common.cuh"
#include "nvtx.cuh"

namespace cilreg {

// status codes returned through the C ABI (0 = success, negative = failure,
// the sign convention of the reference's shared.h:15-38)
enum Status : int {
    OK = 0,
    ERR_CUDA = -1,
    ERR_ARG = -2,
    ERR_NODEV = -3,
    ERR_OOM = -4,
    ERR_CANCELLED = -5,
};

// Host-side fault injection for tests: the next `n` device allocations the
// library makes (scratch and prox sessions) fail as if the device were full.
void inject_allocation_failures(int n);
// true (and one fewer pending failure) when an injected failure is due
bool take_injected_failure();

// record an error (thread-local message, also printed to stderr like the
// reference's CHECK macro) and return the status
int fail(int status, const char* file, int line, const char* fmt, ...);
const char* last_error();

#define CILREG_CUDA(call)                                                                         \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return ::cilreg::fail(e_ == cudaErrorMemoryAllocation ? ::cilreg::ERR_OOM             \
                                                                   : ::cilreg::ERR_CUDA,          \
                                  __FILE__, __LINE__, "code: %d, reason: %s", (int)e_,            \
                                  cudaGetErrorString(e_));                                        \
    } while (0)

#define CILREG_TRY(expr)          \
    do {                          \
        int s_ = (expr);          \
        if (s_ != 0) return s_;   \
    } while (0)

// select the device (checks that one exists) and prepare its memory pool
int use_device(int dev);

// wait for the device's work, then return the memory its pool holds unused
int release_cached(int dev);

// a non-blocking stream owned by the calling host thread for device `dev`
cudaStream_t thread_stream(int dev);

// number of SMs of the current device (cached per device)
int sm_count();

// z-chunk length for a 2.5D streaming kernel: `tiles_xy` CTAs per z chunk,
// `resident` CTAs per SM, `extra` pipeline steps per chunk besides its planes.
// Minimises (rounds of CTAs over the SMs) x (steps per CTA), up to `max_chunk`.
int wave_zchunk(long long tiles_xy, int nz, int resident, int extra, int max_chunk);

// CTAs of `kernel` resident per SM at `threads` threads and no dynamic shared
// memory (at least 1)
template <class K>
int resident_ctas(K kernel, int threads) {
    int r = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, kernel, threads, 0) != cudaSuccess || r <= 0) r = 1;
    return r;
}

// stream-ordered scratch buffers freed when the object is destroyed
class Scratch {
public:
    explicit Scratch(cudaStream_t s) : stream_(s) {}
    ~Scratch();
    // allocate `count` floats (64-byte aligned); returns nullptr on failure
    float* floats(long long count);
    void* bytes(size_t n);
    int status() const { return status_; }

private:
    static const int kMax = 1024;
    cudaStream_t stream_;
    void* ptrs_[kMax] = {};
    int n_ = 0;
    int status_ = 0;
};

// Device-resident stopping control for one regulariser run.
class IterControl {
public:
    IterControl(cudaStream_t s, Scratch& scratch, int iter_total, float epsil, long long max_partials);
    ~IterControl();
    int status() const { return status_; }
    StopCtl* ctl() const { return d_ctl_; }
    double2* partials() const { return d_part_; }
    bool checking() const { return epsil_ != 0.0f; }
    // the reference's test: a check happens at iteration `it` when it % 5 == 0
    bool is_check(int it) const { return epsil_ != 0.0f && (it % 5) == 0; }
    // enqueue the reduction of `nparts` partials for iteration `it`
    int after_check(int it, long long nparts);
    // true when the host may stop enqueueing (the rule has fired on device)
    bool host_should_stop();
    // wait for completion and fill infovector[0..1] (host pointer, may be null)
    int finish(float* infovector, StopCtl* out = nullptr);

private:
    cudaStream_t stream_;
    StopCtl* d_ctl_ = nullptr;
    double2* d_part_ = nullptr;
    StopCtl* h_ring_ = nullptr;  // pinned mirror slots
    cudaEvent_t ev_[4] = {};
    int nev_ = 0, head_ = 0, pending_ = 0;
    float epsil_;
    int status_ = 0;
};

// 1-D helper: grid for n elements with 256-thread CTAs
inline dim3 grid1(long long n) {
    long long b = (n + 255) / 256;
    if (b > 2147483647LL) b = 2147483647LL;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

// Fixed-count iteration loops on small volumes, where a launch costs about as
// much as the kernel: enqueue(it, stream, in_graph) for it in [0, iters),
// with iterations [0, G) captured once into a CUDA graph (in_graph true; then
// tail(stream), which may advance device-side iteration state) and the graph
// replayed while G or more remain, the rest launched directly, all on this
// thread's own stream joined to `s` by events.  Only for loops whose launches
// depend on `it` through `it mod G` (G even) or on device-side state.
struct NoTail {
    int operator()(cudaStream_t) const { return 0; }
};
template <class Enq, class Tail = NoTail>
int run_replayed(int iters, int G, cudaStream_t s, Enq enqueue, Tail tail = Tail());

// Programmatic dependent launch: an iteration kernel launched with
// launch_pdl may be scheduled while the kernel before it in the stream is
// still draining; it runs pdl_wait() before its first memory access (the
// previous grid has then completed and its writes are visible, so both the
// read-after-write and the write-after-read order of ping-pong buffers hold)
// and pdl_trigger() to let its own successor be scheduled early.  Both
// instructions do nothing in a kernel launched without the attribute.
// CILREG_PDL=0 launches normally (A/B checks).  launch_pdl returns the launch
// status and clears it from the thread's error state.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory"); }
bool pdl_enabled();
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args) {
    if (!pdl_enabled()) {
        kernel<<<grid, block, smem, s>>>(args...);
        return cudaGetLastError();
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1] = {};
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, ((KArgs)args)...);
    cudaGetLastError();  // the status is returned; leave no stale error behind
    return e;
}

// process-wide count of kernels this library has launched (for benchmarks)
void note_launch(long long n = 1);
long long launch_count();

// device kernels shared by the drivers (runtime.cu)
// reset a StopCtl (no stop, iters = iter_total, count 0, re 0)
int launch_init_ctl(StopCtl* ctl, int iter_total, cudaStream_t s);
// reduce `nparts` FP64 partials and apply the stopping rule for iteration `it`
int launch_finalize_check(const double2* partials, long long nparts, StopCtl* ctl, float epsil, int it,
                          cudaStream_t s);
// per-volume stopping checks of a batch: slot v reduces part[v][0..n[v]) into ctl[v]
struct CheckSlot {
    const double2* part;
    long long n;
    StopCtl* ctl;
};
int launch_finalize_batch(const CheckSlot* d_slots, int nvol, float epsil, int it, cudaStream_t s);
int launch_init_ctls(StopCtl* const* d_ctls, int nvol, int iter_total, cudaStream_t s);
int launch_fill(float* p, float v, long long n, cudaStream_t s);
int launch_copy(float* dst, const float* src, long long n, cudaStream_t s);
// copy the buffer that holds the final iterate into dst, choosing on device:
// the last written iteration is ctl->iters when stopped, else iter_total-1;
// buffer bufs[(last+1) & 1] holds it (ping-pong with iteration it writing bufs[(it+1)&1]).
int launch_select_pingpong(const StopCtl* ctl, int iter_total, float* const bufs[2], float* dst, long long n,
                           cudaStream_t s);


template <class Enq, class Tail>
int run_replayed(int iters, int G, cudaStream_t s, Enq enqueue, Tail tail) {
    CILREG_RANGE("cilreg graph replay");
    const char* env = getenv("CILREG_GRAPH_REPLAY");  // "0": launch every iteration directly (A/B checks)
    const int reps = (G > 0 && (G % 2) == 0 && !(env && env[0] == '0')) ? iters / G : 0;
    // a stream the caller is capturing records the launches as they are
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const bool capturing = cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
    cudaGetLastError();
    if (reps < 2 || capturing) {
        for (int it = 0; it < iters; it++) CILREG_TRY(enqueue(it, s, false));
        return OK;
    }
    // capture and replay on this thread's own stream t (the caller's may be a
    // default stream, which cannot be captured), ordered after the caller's
    // earlier work and before its later work by two events
    int dev = 0;
    CILREG_CUDA(cudaGetDevice(&dev));
    cudaStream_t t = thread_stream(dev);
    cudaEvent_t ev[2] = {nullptr, nullptr};
    for (int i = 0; i < 2; i++) CILREG_CUDA(cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
    auto finish = [&](int rc) {
        for (int i = 0; i < 2; i++) cudaEventDestroy(ev[i]);
        return rc;
    };
    if (t != s) {
        if (cudaEventRecord(ev[0], s) != cudaSuccess || cudaStreamWaitEvent(t, ev[0], 0) != cudaSuccess)
            return finish(fail(ERR_CUDA, __FILE__, __LINE__, "stream ordering failed"));
    }
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    if (cudaStreamBeginCapture(t, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return finish(fail(ERR_CUDA, __FILE__, __LINE__, "stream capture failed"));
    const long long before = launch_count();
    int rc = OK;
    for (int k = 0; k < G && rc == OK; k++) rc = enqueue(k, t, true);
    if (rc == OK) rc = tail(t);
    const cudaError_t e = cudaStreamEndCapture(t, &g);
    if (rc != OK) {
        if (g) cudaGraphDestroy(g);
        return finish(rc);
    }
    if (e != cudaSuccess) return finish(fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(e)));
    const cudaError_t ei = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return finish(fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(ei)));
    const long long per_graph = launch_count() - before;
    cudaError_t el = cudaSuccess;
    for (int r = 0; r < reps && el == cudaSuccess; r++) el = cudaGraphLaunch(ge, t);
    cudaGraphExecDestroy(ge);  // freed when the queued launches complete
    if (el != cudaSuccess) return finish(fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(el)));
    note_launch(per_graph * (reps - 1));  // the capture counted one replay
    for (int it = reps * G; it < iters && rc == OK; it++) rc = enqueue(it, t, false);
    if (rc != OK) return finish(rc);
    if (t != s) {
        if (cudaEventRecord(ev[1], t) != cudaSuccess || cudaStreamWaitEvent(s, ev[1], 0) != cudaSuccess)
            return finish(fail(ERR_CUDA, __FILE__, __LINE__, "stream ordering failed"));
    }
    return finish(OK);
}


}  // namespace cilreg
