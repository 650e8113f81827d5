// LLT-ROF streaming kernels' launch plan (llt.cu, llt_pair.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct LltPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool pair = false;  // the two-voxels-per-thread kernel (llt_pair.cu)
};

// volumes with nx even and fewer than 2^31 voxels run k_llt_pair (3D) or
// k_llt_pair2d (CILREG_LLT_KERNEL=stream selects k_llt_stream)
bool llt_pair_applies(const Dims& d);
LltPlan llt_pair_plan(const Dims& d);
cudaError_t llt_pair_launch(const LltPlan& T, const float* cur, float* nxt, const float* f, float lam_rof,
                            float lam_llt, float tau, const Dims& d, const StopCtl* ctl, int check,
                            double2* partials, cudaStream_t s);

}  // namespace cilreg
