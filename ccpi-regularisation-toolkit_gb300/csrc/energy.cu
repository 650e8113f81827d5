// TV energy diagnostic (reference: utils.c:60-117, Python TV.py:421
// TV_ENERGY): E = 2 lambda sum |grad U| (+ sum (U - U0)^2 for type 1), forward
// differences with a zero difference at the last index.
//
// One pass over the volume: each term is formed in FP32 exactly as the
// reference forms it (squares and sums without contraction); terms are summed
// in FP64 (per thread, per CTA, then one CTA in a fixed order), so the result
// is deterministic and closer to the exact sum than the reference's
// sequential FP32 accumulator.
#include <math.h>
#include <stdlib.h>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

constexpr int NT = 256;

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

template <bool THREE>
__global__ void __launch_bounds__(NT) k_tv_energy(const float* __restrict__ U, const float* __restrict__ U0,
                                                  float lam2, Dims d, int kz, double2* __restrict__ partials) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    double eg = 0.0, ed = 0.0;
    if (i < d.nx && j < d.ny) {
        const long long dj = (j == d.ny - 1) ? 0 : d.nx;  // zero difference at the last index
        const long long di = (i == d.nx - 1) ? 0 : 1;
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = (long long)k * d.sxy + (long long)j * d.nx + i;
            const float u = __ldg(U + v);
            const float a = __ldg(U + v + dj) - u;  // "x" of the reference: the j axis
            const float b = __ldg(U + v + di) - u;
            float s = __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
            if (THREE) {
                const long long dk = (k == d.nz - 1) ? 0 : d.sxy;
                const float c = __ldg(U + v + dk) - u;
                s = __fadd_rn(s, __fmul_rn(c, c));
            }
            eg += (double)__fmul_rn(lam2, sqrtf(s));
            const float e = u - __ldg(U0 + v);
            ed += (double)__fmul_rn(e, e);
        }
    }
    __shared__ double sa[NT / 32], sb[NT / 32];
    const int tid = threadIdx.x + 32 * threadIdx.y;
    eg = warp_sum_d(eg);
    ed = warp_sum_d(ed);
    if ((tid & 31) == 0) {
        sa[tid >> 5] = eg;
        sb[tid >> 5] = ed;
    }
    __syncthreads();
    if (tid == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < NT / 32; w++) {
            x += sa[w];
            y += sb[w];
        }
        partials[block_slot()] = make_double2(x, y);
    }
}

// one CTA, fixed order: E = gradient term (+ data term) as float
__global__ void __launch_bounds__(NT) k_tv_energy_finish(const double2* __restrict__ partials, long long nparts,
                                                         int type, float* __restrict__ out) {
    __shared__ double sa[NT], sb[NT];
    double x = 0.0, y = 0.0;
    for (long long p = threadIdx.x; p < nparts; p += NT) {
        x += partials[p].x;
        y += partials[p].y;
    }
    sa[threadIdx.x] = x;
    sb[threadIdx.x] = y;
    __syncthreads();
    for (int w = NT / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sa[threadIdx.x] += sa[threadIdx.x + w];
            sb[threadIdx.x] += sb[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = (float)((type == 1) ? sa[0] + sb[0] : sa[0]);
}

// energy of device arrays U, U0 into *e_host (synchronous on stream s)
int tv_energy_run(const float* U, const float* U0, float* e_host, float lambda, int type, const Dims& d,
                  cudaStream_t s) {
    CILREG_RANGE("cilreg TV energy");
    if (type != 1 && type != 2) return fail(ERR_ARG, __FILE__, __LINE__, "type must be 1 or 2 (got %d)", type);
    if (!e_host) return fail(ERR_ARG, __FILE__, __LINE__, "null E_val");
    const Launch3 L = plan_launch(d);
    const long long nparts = num_blocks(L);
    Scratch sc(s);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)nparts);
    float* d_e = sc.floats(1);
    if (!part || !d_e) return sc.status();
    const float lam2 = 2.0f * lambda;  // 2.0f*lambda*sqrtf(...) (utils.c:84)
    if (d.nz > 1)
        k_tv_energy<true><<<L.grid, L.block, 0, s>>>(U, U0, lam2, d, L.kz, part);
    else
        k_tv_energy<false><<<L.grid, L.block, 0, s>>>(U, U0, lam2, d, L.kz, part);
    CILREG_CUDA(cudaGetLastError());
    k_tv_energy_finish<<<1, NT, 0, s>>>(part, nparts, type, d_e);
    CILREG_CUDA(cudaGetLastError());
    note_launch(2);
    CILREG_CUDA(cudaMemcpyAsync(e_host, d_e, sizeof(float), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}

// host arrays: upload, run on CILREG_GPU_DEVICE (default 0); NaN on failure
float energy_host(const float* U, const float* U0, float* E_val, float lambda, int type, int nx, int ny, int nz) {
    const float nan = nanf("");
    if (!U || !U0 || !E_val) {
        fail(ERR_ARG, __FILE__, __LINE__, "null pointer");
        return nan;
    }
    E_val[0] = nan;
    if (check_dims(nx, ny, nz) != 0) return nan;
    const char* e = getenv("CILREG_GPU_DEVICE");
    const int dev = e ? atoi(e) : 0;
    if (use_device(dev) != 0) return nan;
    cudaStream_t s = thread_stream(dev);
    const Dims d = make_dims(nx, ny, nz < 1 ? 1 : nz);
    float out = nan;
    int rc;
    {
        Scratch io(s);
        float* du = io.floats(d.n);
        float* du0 = io.floats(d.n);
        if (!du || !du0) return nan;
        const size_t bytes = sizeof(float) * (size_t)d.n;
        if (cudaMemcpyAsync(du, U, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(du0, U0, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            fail(ERR_CUDA, __FILE__, __LINE__, "host to device copy failed");
            return nan;
        }
        rc = tv_energy_run(du, du0, &out, lambda, type, d, s);
    }
    if (rc != OK) return nan;
    E_val[0] = out;
    return out;
}

}  // namespace
}  // namespace cilreg

using namespace cilreg;

extern "C" {

float TV_energy2D(float* U, float* U0, float* E_val, float lambda, int type, int dimX, int dimY) {
    return energy_host(U, U0, E_val, lambda, type, dimX, dimY, 1);
}

float TV_energy3D(float* U, float* U0, float* E_val, float lambda, int type, int dimX, int dimY, int dimZ) {
    return energy_host(U, U0, E_val, lambda, type, dimX, dimY, dimZ);
}

int cilreg_tv_energy_dev(const float* d_u, const float* d_u0, float* E_val, float lambda, int type, int dimX,
                         int dimY, int dimZ, void* stream) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    if (!d_u || !d_u0) return fail(ERR_ARG, __FILE__, __LINE__, "null device pointer");
    return tv_energy_run(d_u, d_u0, E_val, lambda, type, make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ),
                         (cudaStream_t)stream);
}

}  // extern "C"
