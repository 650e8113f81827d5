// Self-test of the bounded waits of the kernels that stage their inputs by
// tensor copies (tma_ring.cuh).  A wait on a stage's mbarrier gives up after
// a fixed number of tries and the kernel records the failure instead of
// spinning forever; this probe makes such a wait run out on purpose, without
// any fault: one CTA arms an mbarrier for 16 bytes that no copy delivers (no
// copy is issued, so nothing is in flight when the kernel returns), waits on
// it with the same helper the kernels use, and writes whether the wait gave
// up.  The host reads that status and checks that the context still runs
// work afterwards.
#include "pair.cuh"
#include "runtime.cuh"
#include "tma_ring.cuh"

namespace cilreg {
namespace {

// *out: 1 if the wait saw the phase complete (it must not), 2 if it ran out
__global__ void k_wait_limit_probe(int* out) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tma::mbar_init(&bar);
        tma::mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) tma::mbar_expect(&bar, 16);  // arrival done, 16 bytes outstanding
    __syncthreads();
    const bool landed = tma::wait_stage(&bar, 0);
    __syncthreads();
    if (threadIdx.x == 0) *out = landed ? 1 : 2;
}

__global__ void k_set_int(int* p, int v) { *p = v; }

// rcp2 (pair.cuh) and CUDA's IEEE reciprocal of every x
__global__ void k_reciprocal_probe(const float* x, float* approx, float* ieee, long long n) {
    const long long i = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= n) return;
    const float a = x[i], b = (i + 1 < n) ? x[i + 1] : 1.0f;
    const float2 r = pair::rcp2(make_float2(a, b));
    approx[i] = r.x;
    ieee[i] = __frcp_rn(a);
    if (i + 1 < n) {
        approx[i + 1] = r.y;
        ieee[i + 1] = __frcp_rn(b);
    }
}

}  // namespace
}  // namespace cilreg

extern "C" int cilreg_selftest_wait_limit(int gpu_device, int* ran_out) {
    using namespace cilreg;
    if (!ran_out) return fail(ERR_ARG, __FILE__, __LINE__, "null ran_out");
    *ran_out = 0;
    CILREG_TRY(use_device(gpu_device));
    cudaStream_t s = thread_stream(gpu_device);
    Scratch sc(s);
    int* d = (int*)sc.bytes(sizeof(int));
    if (!d) return sc.status();
    CILREG_CUDA(cudaMemsetAsync(d, 0, sizeof(int), s));
    k_wait_limit_probe<<<1, 32, 0, s>>>(d);
    CILREG_CUDA(cudaGetLastError());
    int h = 0;
    CILREG_CUDA(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (h != 1 && h != 2) return fail(ERR_CUDA, __FILE__, __LINE__, "the wait probe wrote %d", h);
    // the context still runs work after the wait gave up
    k_set_int<<<1, 1, 0, s>>>(d, 7);
    CILREG_CUDA(cudaGetLastError());
    int after = 0;
    CILREG_CUDA(cudaMemcpyAsync(&after, d, sizeof(int), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (after != 7) return fail(ERR_CUDA, __FILE__, __LINE__, "no work ran after the wait probe");
    *ran_out = (h == 2) ? 1 : 0;
    return OK;
}

extern "C" int cilreg_selftest_reciprocal(int gpu_device, const float* x, float* approx, float* ieee,
                                          long long n) {
    using namespace cilreg;
    if (!x || !approx || !ieee || n < 1 || n > (1LL << 30))
        return fail(ERR_ARG, __FILE__, __LINE__, "bad reciprocal probe arguments (n = %lld)", n);
    CILREG_TRY(use_device(gpu_device));
    cudaStream_t s = thread_stream(gpu_device);
    Scratch sc(s);
    float* d = sc.floats(3 * n);
    if (!d) return sc.status();
    CILREG_CUDA(cudaMemcpyAsync(d, x, sizeof(float) * n, cudaMemcpyHostToDevice, s));
    const long long pairs = (n + 1) / 2;
    k_reciprocal_probe<<<(unsigned)((pairs + 255) / 256), 256, 0, s>>>(d, d + n, d + 2 * n, n);
    CILREG_CUDA(cudaGetLastError());
    CILREG_CUDA(cudaMemcpyAsync(approx, d + n, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaMemcpyAsync(ieee, d + 2 * n, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}
