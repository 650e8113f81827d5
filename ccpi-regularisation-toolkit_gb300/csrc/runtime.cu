// Host runtime: errors, devices, per-thread streams, scratch, stopping control.
#include "runtime.cuh"

#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

namespace cilreg {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void note_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

int fail(int status, const char* file, int line, const char* fmt, ...) {
    char msg[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    const char* base = strrchr(file, '/');
    snprintf(g_err, sizeof(g_err), "Error: %s:%d, %s", base ? base + 1 : file, line, msg);
    fprintf(stderr, "%s\n", g_err);
    return status;
}

const char* last_error() { return g_err; }

// ---------------------------------------------------------------------------
static std::once_flag g_pool_once[64];

int use_device(int dev) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        return fail(ERR_NODEV, __FILE__, __LINE__, "No CUDA devices found");
    }
    if (dev < 0 || dev >= count) {
        return fail(ERR_ARG, __FILE__, __LINE__, "gpu_device %d out of range (0..%d)", dev, count - 1);
    }
    CILREG_CUDA(cudaSetDevice(dev));
    if (dev < 64) {
        std::call_once(g_pool_once[dev], [dev]() {
            // keep freed scratch cached in the stream-ordered pool so that
            // repeated calls do not remap device memory
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t thr = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            }
        });
    }
    return OK;
}

int release_cached(int dev) {
    CILREG_TRY(use_device(dev));
    CILREG_CUDA(cudaDeviceSynchronize());
    cudaMemPool_t pool;
    CILREG_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    CILREG_CUDA(cudaMemPoolTrimTo(pool, 0));
    return OK;
}

cudaStream_t thread_stream(int dev) {
    struct Streams {
        cudaStream_t s[64] = {};
        ~Streams() {
            // streams die with the context at process exit; nothing to do
        }
    };
    static thread_local Streams ts;
    if (dev < 0 || dev >= 64) return 0;
    if (!ts.s[dev]) {
        if (cudaStreamCreateWithFlags(&ts.s[dev], cudaStreamNonBlocking) != cudaSuccess) ts.s[dev] = 0;
    }
    return ts.s[dev];
}

int sm_count() {
    static std::atomic<int> cache[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

bool pdl_enabled() {
    const char* e = getenv("CILREG_PDL");
    return !(e && e[0] == '0');
}

int wave_zchunk(long long tiles_xy, int nz, int resident, int extra, int max_chunk) {
    if (nz <= 1) return 1;
    if (max_chunk > nz) max_chunk = nz;
    if (const char* e = getenv("CILREG_STREAM_ZCHUNK")) {
        const int v = atoi(e);
        if (v > 0) return v < nz ? v : nz;
    }
    const long long slots = (long long)sm_count() * (resident > 0 ? resident : 1);
    int best = max_chunk;
    double best_cost = -1.0;
    for (int zc = max_chunk; zc >= 8 || zc == max_chunk; zc--) {
        const long long blocks = tiles_xy * ((nz + zc - 1) / zc);
        const long long rounds = (blocks + slots - 1) / slots;
        const double cost = (double)rounds * (double)(zc + extra);
        if (best_cost < 0 || cost < best_cost * 0.995) {  // prefer longer chunks on ties
            best_cost = cost;
            best = zc;
        }
        if (zc <= 1) break;
    }
    return best;
}

// ---------------------------------------------------------------------------
Scratch::~Scratch() {
    for (int i = 0; i < n_; i++)
        if (ptrs_[i]) cudaFreeAsync(ptrs_[i], stream_);
}

namespace {
std::atomic<int> g_injected_failures{0};
}

void inject_allocation_failures(int n) { g_injected_failures.store(n < 0 ? 0 : n); }

bool take_injected_failure() {
    int v = g_injected_failures.load();
    while (v > 0)
        if (g_injected_failures.compare_exchange_weak(v, v - 1)) return true;
    return false;
}

void* Scratch::bytes(size_t n) {
    if (n_ >= kMax) {
        status_ = fail(ERR_ARG, __FILE__, __LINE__, "scratch slot table exhausted");
        return nullptr;
    }
    if (take_injected_failure()) {
        status_ = fail(ERR_OOM, __FILE__, __LINE__, "scratch allocation of %zu bytes failed: injected failure", n);
        return nullptr;
    }
    void* p = nullptr;
    const size_t sz = n < 64 ? 64 : n;
    cudaError_t e = cudaMallocAsync(&p, sz, stream_);
    // the pool keeps freed scratch; when the device is full, hand the unused
    // part back first (then also what this stream's earlier calls freed) and
    // retry, so that other allocators on the device are not starved by it
    for (int attempt = 0; e == cudaErrorMemoryAllocation && attempt < 2; attempt++) {
        cudaGetLastError();
        if (attempt == 1) cudaStreamSynchronize(stream_);
        int dev = 0;
        cudaMemPool_t pool;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
            cudaMemPoolTrimTo(pool, 0);
        e = cudaMallocAsync(&p, sz, stream_);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        status_ = fail(e == cudaErrorMemoryAllocation ? ERR_OOM : ERR_CUDA, __FILE__, __LINE__,
                       "scratch allocation of %zu bytes failed: %s", n, cudaGetErrorString(e));
        return nullptr;
    }
    ptrs_[n_++] = p;
    return p;
}

float* Scratch::floats(long long count) { return (float*)bytes((size_t)(count < 1 ? 1 : count) * sizeof(float)); }

// ---------------------------------------------------------------------------
__global__ void k_init_ctl(StopCtl* c, int iters) {
    c->stop = 0;
    c->iters = iters;
    c->count = 0;
    c->re = 0.0f;
}

// Deterministic reduction of the per-CTA FP64 partials, then the stopping
// rule.  One CTA of 1024 threads; fixed assignment of partials to threads.
__global__ void __launch_bounds__(1024) k_finalize_check(const double2* __restrict__ part, long long nparts,
                                                          StopCtl* ctl, float epsil, int it) {
    if (ctl->stop) return;
    double a = 0.0, b = 0.0;
    for (long long p = threadIdx.x; p < nparts; p += 1024) {
        double2 v = part[p];
        a += v.x;
        b += v.y;
    }
    __shared__ double sa[32], sb[32];
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x < 32) {
        a = warp_sum(sa[threadIdx.x]);
        b = warp_sum(sb[threadIdx.x]);
        if (threadIdx.x == 0) {
            float re = sqrtf((float)a) / sqrtf((float)b);
            ctl->re = re;
            if (re < epsil) ctl->count += 1;
            if (ctl->count > 3) {
                ctl->stop = 1;
                ctl->iters = it;
            }
        }
    }
}

namespace {

// pinned mirrors of the stop control, kept per host thread and reused across
// calls (cudaMallocHost / cudaFreeHost per call cost tens of microseconds and
// the free can wait for the device); a small stack, since calls may nest
struct PinnedMirrors {
    std::vector<StopCtl*> free_list;
    ~PinnedMirrors() {
        // process exit: the CUDA context may already be gone, so leave them
    }
};
thread_local PinnedMirrors t_mirrors;

StopCtl* take_mirror() {
    if (!t_mirrors.free_list.empty()) {
        StopCtl* p = t_mirrors.free_list.back();
        t_mirrors.free_list.pop_back();
        return p;
    }
    StopCtl* p = nullptr;
    if (cudaMallocHost((void**)&p, sizeof(StopCtl) * 5) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void give_mirror(StopCtl* p) {
    if (p) t_mirrors.free_list.push_back(p);
}

}  // namespace

IterControl::IterControl(cudaStream_t s, Scratch& scratch, int iter_total, float epsil, long long max_partials)
    : stream_(s), epsil_(epsil) {
    d_ctl_ = (StopCtl*)scratch.bytes(sizeof(StopCtl));
    if (!d_ctl_) { status_ = scratch.status(); return; }
    if (epsil != 0.0f) {
        d_part_ = (double2*)scratch.bytes(sizeof(double2) * (size_t)(max_partials < 1 ? 1 : max_partials));
        if (!d_part_) { status_ = scratch.status(); return; }
    }
    k_init_ctl<<<1, 1, 0, s>>>(d_ctl_, iter_total);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { status_ = fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(e)); return; }
    if (!(h_ring_ = take_mirror())) {
        status_ = fail(ERR_CUDA, __FILE__, __LINE__, "pinned allocation failed");
        return;
    }
    memset(h_ring_, 0, sizeof(StopCtl) * 5);
    if (epsil != 0.0f) {
        for (int i = 0; i < 4; i++) {
            if (cudaEventCreateWithFlags(&ev_[i], cudaEventDisableTiming) != cudaSuccess) {
                status_ = fail(ERR_CUDA, __FILE__, __LINE__, "event creation failed");
                return;
            }
            nev_++;
        }
    }
}

IterControl::~IterControl() {
    // error paths return before finish(): drain the stream before releasing
    // the pinned mirror that pending copies may still target
    if (h_ring_) {
        cudaStreamSynchronize(stream_);
        give_mirror(h_ring_);
    }
    for (int i = 0; i < nev_; i++) cudaEventDestroy(ev_[i]);
}

int IterControl::after_check(int it, long long nparts) {
    k_finalize_check<<<1, 1024, 0, stream_>>>(d_part_, nparts, d_ctl_, epsil_, it);
    note_launch();
    CILREG_CUDA(cudaGetLastError());
    // mirror the control block to pinned memory and remember the event, so the
    // host can stop enqueueing a few iterations after the rule fires
    int slot = head_ % 4;
    CILREG_CUDA(cudaMemcpyAsync(&h_ring_[slot], d_ctl_, sizeof(StopCtl), cudaMemcpyDeviceToHost, stream_));
    CILREG_CUDA(cudaEventRecord(ev_[slot], stream_));
    head_++;
    if (pending_ < 4) pending_++;
    return OK;
}

bool IterControl::host_should_stop() {
    if (epsil_ == 0.0f || pending_ == 0) return false;
    // keep up to two checks (about ten iterations) in flight; wait on older ones
    while (pending_ > 2) {
        int slot = (head_ - pending_) % 4;
        cudaEventSynchronize(ev_[slot]);
        pending_--;
        if (h_ring_[slot].stop) return true;
    }
    int slot = (head_ - pending_) % 4;
    if (cudaEventQuery(ev_[slot]) == cudaSuccess) {
        pending_--;
        if (h_ring_[slot].stop) return true;
    }
    return false;
}

int IterControl::finish(float* infovector, StopCtl* out) {
    if (!h_ring_) return status_ ? status_ : ERR_CUDA;
    CILREG_CUDA(cudaMemcpyAsync(&h_ring_[4], d_ctl_, sizeof(StopCtl), cudaMemcpyDeviceToHost, stream_));
    CILREG_CUDA(cudaStreamSynchronize(stream_));
    StopCtl c = h_ring_[4];
    if (infovector) {
        infovector[0] = (float)c.iters;
        infovector[1] = c.re;
    }
    if (out) *out = c;
    for (int i = 0; i < nev_; i++) cudaEventDestroy(ev_[i]);
    nev_ = 0;
    give_mirror(h_ring_);
    h_ring_ = nullptr;
    return OK;
}

// ---------------------------------------------------------------------------
__global__ void k_fill(float* p, float v, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) p[i] = v;
}

__global__ void k_copy(float* __restrict__ d, const float* __restrict__ s, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) d[i] = s[i];
}

__global__ void k_select_copy(const StopCtl* ctl, int iter_total, const float* b0, const float* b1, float* dst,
                              long long n) {
    int last = ctl->stop ? ctl->iters : iter_total - 1;
    const float* src = ((last + 1) & 1) ? b1 : b0;
    if (src == dst) return;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) dst[i] = src[i];
}

static dim3 grid_stride_blocks(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152LL * 16) b = 152LL * 16;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

// one CTA per volume; the same fixed-order reduction as k_finalize_check
__global__ void __launch_bounds__(1024) k_finalize_batch(const CheckSlot* __restrict__ slots, float epsil, int it) {
    const CheckSlot c = slots[blockIdx.x];
    if (c.ctl->stop) return;
    double a = 0.0, b = 0.0;
    for (long long p = threadIdx.x; p < c.n; p += 1024) {
        double2 v = c.part[p];
        a += v.x;
        b += v.y;
    }
    __shared__ double sa[32], sb[32];
    a = warp_sum(a);
    b = warp_sum(b);
    if ((threadIdx.x & 31) == 0) { sa[threadIdx.x >> 5] = a; sb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x < 32) {
        a = warp_sum(sa[threadIdx.x]);
        b = warp_sum(sb[threadIdx.x]);
        if (threadIdx.x == 0) {
            float re = sqrtf((float)a) / sqrtf((float)b);
            c.ctl->re = re;
            if (re < epsil) c.ctl->count += 1;
            if (c.ctl->count > 3) {
                c.ctl->stop = 1;
                c.ctl->iters = it;
            }
        }
    }
}

__global__ void k_init_ctls(StopCtl* const* ctls, int nvol, int iters) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nvol) {
        ctls[v]->stop = 0;
        ctls[v]->iters = iters;
        ctls[v]->count = 0;
        ctls[v]->re = 0.0f;
    }
}

int launch_finalize_batch(const CheckSlot* d_slots, int nvol, float epsil, int it, cudaStream_t s) {
    k_finalize_batch<<<nvol, 1024, 0, s>>>(d_slots, epsil, it);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    return OK;
}

int launch_init_ctls(StopCtl* const* d_ctls, int nvol, int iter_total, cudaStream_t s) {
    k_init_ctls<<<(nvol + 127) / 128, 128, 0, s>>>(d_ctls, nvol, iter_total);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    return OK;
}

int launch_init_ctl(StopCtl* ctl, int iter_total, cudaStream_t s) {
    k_init_ctl<<<1, 1, 0, s>>>(ctl, iter_total);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    return OK;
}

int launch_finalize_check(const double2* partials, long long nparts, StopCtl* ctl, float epsil, int it,
                          cudaStream_t s) {
    k_finalize_check<<<1, 1024, 0, s>>>(partials, nparts, ctl, epsil, it);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    return OK;
}

int launch_fill(float* p, float v, long long n, cudaStream_t s) {
    k_fill<<<grid_stride_blocks(n), 256, 0, s>>>(p, v, n);
    note_launch();
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int launch_copy(float* dst, const float* src, long long n, cudaStream_t s) {
    k_copy<<<grid_stride_blocks(n), 256, 0, s>>>(dst, src, n);
    note_launch();
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int launch_select_pingpong(const StopCtl* ctl, int iter_total, float* const bufs[2], float* dst, long long n,
                           cudaStream_t s) {
    k_select_copy<<<grid_stride_blocks(n), 256, 0, s>>>(ctl, iter_total, bufs[0], bufs[1], dst, n);
    note_launch();
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace cilreg
