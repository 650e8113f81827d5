// Shared device/host infrastructure for the GB300 regulariser kernels.
//
// Layout: every array is a C-ordered float32 volume of nz slices of ny rows of
// nx voxels (nx fastest), linear index (nx*ny)*k + nx*j + i, exactly the
// reference's convention (src/Python/ccpi/filters/TV.py:37-39,
// src/Core/regularisers_CPU/FGP_TV_core.c:228).  A 2D image is nz == 1.
//
// Stopping rule (all seven algorithms, e.g. FGP_TV_core.c:142-153): when
// epsil != 0 and iter % 5 == 0, re = ||U - U_prev|| / ||U||; count++ when
// re < epsil; stop when count > 3 (cumulative).  Here the two sums are FP64
// per-CTA partials reduced in a fixed order by one finalize kernel, which
// updates a device-resident StopCtl.  Every iteration kernel first reads
// StopCtl::stop and returns at once when it is set, so the host can enqueue
// iterations without waiting for the decision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace cilreg {

struct StopCtl {
    int stop;     // 1 once the stopping rule has fired
    int iters;    // infovector[0]: the break index, or the requested count
    int count;    // cumulative number of checks with re < epsil
    float re;     // infovector[1]: the last relative change
};

struct Dims {
    int nx, ny, nz;
    long long sxy;  // nx*ny
    long long n;    // nx*ny*nz
};

inline Dims make_dims(int nx, int ny, int nz) {
    Dims d;
    d.nx = nx; d.ny = ny; d.nz = nz;
    d.sxy = (long long)nx * ny;
    d.n = d.sxy * nz;
    return d;
}

// mirrored neighbours (symmetric/Neumann boundary of the reference):
// hi(i) = i+1, or i-1 at the last index; lo(i) = i-1, or i+1 at index 0.
// On an axis of length 1 both return the voxel itself.
__device__ __forceinline__ int nb_hi(int i, int n) { return (n == 1) ? 0 : ((i + 1 >= n) ? i - 1 : i + 1); }
__device__ __forceinline__ int nb_lo(int i, int n) { return (n == 1) ? 0 : ((i - 1 < 0) ? i + 1 : i - 1); }

__device__ __forceinline__ long long vid(const Dims& d, int i, int j, int k) {
    return (long long)k * d.sxy + (long long)j * d.nx + i;
}

__device__ __forceinline__ float ldg(const float* p, long long v) { return __ldg(p + v); }

__device__ __forceinline__ float sgnf(float x) { return (float)((x > 0.0f) - (x < 0.0f)); }

// p / max(|p|, 1), the anisotropic projection of FGP and PD (utils.c:198-210),
// with the IEEE quotient's value and no division: p itself for |p| <= 1, the
// exact quotient +-1 for finite |p| > 1, NaN for an infinite p (and p - p is
// NaN for a NaN p too)
__device__ __forceinline__ float unit_clip(float p) {
    const float a = fabsf(p);
    return (a <= 1.0f) ? p : ((a <= 3.4028234664e38f) ? copysignf(1.0f, p) : p - p);
}

// flags between CTAs of one launch: an acquire load and a release store at
// GPU scope
__device__ __forceinline__ int ld_acquire_gpu(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(int* p, int v) {
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---------------------------------------------------------------------------
// block-level FP64 pair reduction -> one double2 partial per CTA
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// All threads of the block must call this (no early return before it).
// Each thread passes FP32 sums of its own (at most a few dozen) voxels; the
// block and grid levels add in FP64.  GB300's FP64 rate is a small fraction
// of its FP32 rate, so per-voxel accumulation stays in FP32.
template <int NTHREADS>
__device__ __forceinline__ void block_pair_partial(float fa, float fb, double2* partials, long long slot) {
    __shared__ double sa[NTHREADS / 32], sb[NTHREADS / 32];
    const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
    double a = warp_sum((double)fa);
    double b = warp_sum((double)fb);
    if ((tid & 31) == 0) { sa[tid >> 5] = a; sb[tid >> 5] = b; }
    __syncthreads();
    if (tid < 32) {
        a = (tid < NTHREADS / 32) ? sa[tid] : 0.0;
        b = (tid < NTHREADS / 32) ? sb[tid] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
        if (tid == 0) partials[slot] = make_double2(a, b);
    }
}

// launch helpers --------------------------------------------------------------
struct Launch3 {
    dim3 grid, block;
    int kz;  // z-slices handled by one CTA
};

// CTA of 32 x 8 threads; each thread walks kz slices so that large volumes
// need O(10^4..10^5) CTAs (one FP64 partial each), not one CTA per slice.
inline Launch3 plan_launch(const Dims& d) {
    Launch3 L;
    L.block = dim3(32, 8, 1);
    L.kz = (d.nz >= 64) ? 8 : ((d.nz >= 8) ? 4 : 1);
    L.grid = dim3((d.nx + 31) / 32, (d.ny + 7) / 8, (d.nz + L.kz - 1) / L.kz);
    return L;
}

inline long long num_blocks(const Launch3& L) {
    return (long long)L.grid.x * L.grid.y * L.grid.z;
}

__device__ __forceinline__ long long block_slot() {
    return (long long)blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
}

}  // namespace cilreg
