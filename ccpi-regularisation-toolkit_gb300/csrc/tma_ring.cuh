// Staging of input planes by the Tensor Memory Accelerator for the 2.5D
// streaming kernels (used by fgp_tma.cu and tgv_fused_tma.cu), and the
// per-thread asynchronous copies (used by rof_tiled.cu and tgv_fused_tma.cu).
//
// A kernel keeps a ring of STAGES shared-memory stages, each holding the
// tile's box of every input array for one plane, and one mbarrier per stage.
// One thread issues a plane's tensor copies (cp.async.bulk.tensor, 3D tile
// mode) onto its stage's mbarrier with the stage's byte count; every thread
// waits on the mbarrier (bounded) before reading its own voxels.  Boxes are
// BOXX x BY floats starting at the tile's first x rounded down to a multiple
// of 4 (a tensor copy's x origin must be 16-byte aligned); out-of-volume
// elements arrive as zeros.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "runtime.cuh"

namespace cilreg {
namespace tma {

constexpr int BOXX = 36;  // box width: a 32-thread row plus up to 3 columns of alignment
constexpr long long WAIT_LIMIT = 1LL << 20;  // tries of a suspending wait: about a second

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// generic-proxy accesses of a stage before the tensor copies that refill it
__device__ __forceinline__ void proxy_fence() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void load_box(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(smem_addr(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
        : "memory");
}
// x origin of a box that covers [xf, xf + 32): xf rounded down to a multiple of 4
__device__ __forceinline__ int box_x0(int xf) { return xf - (((xf % 4) + 4) % 4); }

// bounded wait for `use`-th completion of a stage's mbarrier; false if the
// limit ran out (the caller records the failure and carries on without waiting)
__device__ __forceinline__ bool wait_stage(uint64_t* bar, int use) {
    const uint32_t parity = (uint32_t)(use & 1);
    for (long long t = 0; t < WAIT_LIMIT; t++)
        if (mbar_try(bar, parity)) return true;
    return false;
}

// per-thread asynchronous global -> shared copies of 4 bytes (cp.async,
// sm_80+), grouped per plane; a thread waits for its own groups only
__device__ __forceinline__ void cp_async4(float* sdst, const float* gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_addr(sdst)), "l"(gsrc) : "memory");
}
// ... of 8 bytes (both addresses 8-byte aligned)
__device__ __forceinline__ void cp_async8(float* sdst, const float* gsrc) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_addr(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// host: cuTensorMapEncodeTiled from the driver (null if unavailable)
using EncodeFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                              const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
inline EncodeFn encoder() {
    static EncodeFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        cudaGetLastError();
        return (EncodeFn)p;
    }();
    return fn;
}

// a 3D volume qualifies when its row pitch is a multiple of 16 bytes
inline bool volume_ok(const Dims& d) { return d.nz > 1 && d.nx % 4 == 0 && encoder() != nullptr; }

// tensor map of one float32 volume with boxes of BOXX x boxy x 1; false when
// the base address is not 16-byte aligned or the driver refuses the map
inline bool encode(CUtensorMap* map, const float* base, const Dims& d, int boxy) {
    if (((uintptr_t)base & 15) != 0 || !encoder()) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)d.nx, (cuuint64_t)d.ny, (cuuint64_t)d.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)d.nx * sizeof(float), (cuuint64_t)d.sxy * sizeof(float)};
    const cuuint32_t box[3] = {(cuuint32_t)BOXX, (cuuint32_t)boxy, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return encoder()(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tma
}  // namespace cilreg
