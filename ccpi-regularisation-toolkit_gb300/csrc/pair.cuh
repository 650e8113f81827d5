// Helpers of the kernels that hold two voxels per thread along x (x even):
// paired FP32 arithmetic (FADD2/FMUL2/FFMA2 of sm_100 and later, each
// component rounded exactly as the scalar instruction), 8-byte shared-memory
// accesses, integral-constant step indices, and the tile geometry shared by
// those kernels.
#pragma once

#include <type_traits>

#include "runtime.cuh"

namespace cilreg {
namespace pair {

constexpr int PX = 16;      // threads along x, one voxel pair each
constexpr int TW = 2 * PX;  // tile points along x
constexpr int OXP = TW - 2; // updated voxels along x (one-voxel halo)

// x origin of tile bx: even, so that the pairs of a tile are the volume's
// pairs; the first tile starts two voxels before the volume
__device__ __forceinline__ int tile_x0(int bx) { return bx * OXP - 2; }
// tiles along x that cover nx voxels with one-voxel halos
inline int tiles_x(int nx) { return (nx + OXP) / OXP; }

template <int V>
using Ic = std::integral_constant<int, V>;
template <int V>
__device__ __forceinline__ constexpr int ival(Ic<V>) {
    return V;
}
__device__ __forceinline__ int ival(int v) { return v; }

__device__ __forceinline__ float2 splat(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
// 1/x per component, for normal x whose reciprocal is normal: the hardware's
// approximate reciprocal (PTX rcp.approx.ftz.f32) refined by one
// Newton-Raphson step r + r (1 - x r), whose error term is formed exactly by
// the fused multiply-add; the step issues paired.
__device__ __forceinline__ float2 rcp2(float2 x) {
    float2 r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.x) : "f"(x.x));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.y) : "f"(x.y));
    return fma2(r, fma2(neg2(x), r, make_float2(1.0f, 1.0f)), r);
}

// 8-byte access of a pair (shared or global memory, 8-byte aligned)
__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

__device__ __forceinline__ bool aligned8(const void* p) { return ((uintptr_t)p & 7) == 0; }
inline bool host_aligned8(const void* p) { return ((uintptr_t)p & 7) == 0; }

// plane held by ring slot of plane k: planes beyond the volume hold its
// mirrored planes (-1 -> 1, nz -> nz-2, the reference's k mirrors), planes
// further out are clamped into the volume
__device__ __forceinline__ int ring_plane(int k, int nz) {
    k = (k < 0) ? -k : k;
    k = (k < nz) ? k : max(2 * nz - 2 - k, 0);
    return min(k, nz - 1);
}

// store an updated pair: one 8-byte store where both voxels are updated, one
// 4-byte store at the tile and volume edges (predicated, no branch)
template <bool ALIGNED>
__device__ __forceinline__ void store_pair(float* dst, float2 v, bool vx, bool vy) {
    if (ALIGNED) {
        if (vx && vy) st2(dst, v);
        if (vx && !vy) dst[0] = v.x;
        if (vy && !vx) dst[1] = v.y;
    } else {
        if (vx) dst[0] = v.x;
        if (vy) dst[1] = v.y;
    }
}

}  // namespace pair
}  // namespace cilreg
