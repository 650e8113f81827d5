// Non-linear diffusion: the edge-stopping function shared by the per-voxel
// kernel (ndf.cu) and the 2.5D streaming kernel (ndf_tiled.cu), and the
// streaming kernel's entry points.
#pragma once

#include "runtime.cuh"

namespace cilreg {

// edge-stopping function of one neighbour difference (Diffusion_core.c:315-404)
// (e / sigma is formed as e * isg, isg = 1/sigma from the host: one multiply
// instead of an IEEE division, within 1 ulp of the reference's quotient)
template <int PEN>
__device__ __forceinline__ float flux(float e, float sg, float isg) {
    if (PEN == 0) return e;  // linear diffusion (sigma == 0)
    if (PEN == 1) return (fabsf(e) > sg) ? copysignf(1.0f, e) : e * isg;
    if (PEN == 2) {
        const float r = e * isg;
        return e * __frcp_rn(1.0f + r * r);
    }
    if (PEN == 3) {
        if (fabsf(e) <= sg) {
            const float r = e * isg;
            const float w = 1.0f - r * r;
            return e * (w * w);
        }
        return 0.0f;
    }
    if (PEN == 4) return (fabsf(e) > sg) ? 0.0f : e;
    // PEN == 5
    if (fabsf(e) <= 2.0f * sg) return (fabsf(e) > sg) ? copysignf(1.0f, e) : e * isg;
    return 0.0f;
}

// sg >= 0 (the host clamps it), so |e| > sg means e != 0 and the sign of e is
// a sign copy (the reference's sign function, which is 0 only at e == 0).
// Every penalty is odd (flux(-e) == -flux(e) bit for bit: the sign enters
// only through e itself or its sign copy), so the flux through a face can be formed
// once and used with opposite signs by the two voxels that share it.

struct NdfPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool use = false;   // false: the per-voxel kernel of ndf.cu runs instead
    bool pair = false;  // the two-voxels-per-thread kernel (ndf_pair.cu)
};

// the plan of the kernel that runs for `d`: volumes and images with nx even
// and fewer than 2^31 voxels run k_ndf_pair (3D) or k_ndf_pair2d, others
// below 2^31 voxels k_ndf_stream (CILREG_NDF_KERNEL=stream or simple select a
// one-voxel kernel)
NdfPlan ndf_stream_plan(const Dims& d);
bool ndf_pair_applies(const Dims& d);
NdfPlan ndf_pair_plan(const Dims& d);
int ndf_pair_step(const NdfPlan& T, int pen, const float* cur, float* nxt, const float* f, float lam, float sg,
                  float isg, float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials,
                  cudaStream_t s);
int ndf_stream_step(const NdfPlan& T, int pen, const float* cur, float* nxt, const float* f, float lam, float sg,
                    float isg, float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials,
                    cudaStream_t s);

}  // namespace cilreg
