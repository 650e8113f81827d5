// Split-Bregman TV: the two Jacobi sweeps of one outer iteration fused into
// one 2.5D streaming kernel (sb_tiled.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct SbSweepArgs {
    const float* u;        // U at the start of the outer iteration
    float* u2;             // U after the second sweep
    const float* f;
    const float* dd[3];    // split variables D (read only here)
    const float* bb[3];    // Bregman variables B (read only here)
    float lambda, mu, norm;
};

// one whole outer iteration k >= 1 (k_sb_fused): D^k and B^k formed on the
// fly from U^k and B^{k-1}; writes U^{k+1} and B^k
struct SbFusedArgs {
    const float* u;        // U^k
    float* u2;             // U^{k+1}
    const float* f;
    const float* bp[3];    // B^{k-1}
    float* bn[3];          // B^k (distinct buffers: a neighbouring tile still reads B^{k-1})
    float lambda, mu, norm, dlam;
};

struct SbPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool use = false;  // false: the per-sweep kernels of sb.cu run instead
};

SbPlan sb_sweep2_plan(const Dims& d);
// both sweeps; on a check iteration one FP64 partial of (|U2 - U1|^2, |U2|^2)
// per CTA (SbPlan::nblocks of them)
int sb_sweep2_step(const SbPlan& T, const SbSweepArgs& a, const Dims& d, const StopCtl* ctl, int check,
                   double2* partials, cudaStream_t s);
// one outer iteration k >= 1 with the shrinkage fused in (same tiling and
// partial slots as sb_sweep2_step)
int sb_fused_step(const SbPlan& T, const SbFusedArgs& a, bool aniso, const Dims& d, const StopCtl* ctl, int check,
                  double2* partials, cudaStream_t s);

}  // namespace cilreg
