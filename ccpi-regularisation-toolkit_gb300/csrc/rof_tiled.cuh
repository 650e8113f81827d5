// 2.5D streaming ROF-TV iteration (rof_tiled.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct RofPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
};

RofPlan rof_tiled_plan(const Dims& d);

// one iteration: reads cur, writes nxt; on a check iteration one FP64 partial
// per CTA (RofPlan::nblocks of them)
int rof_tiled_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                   float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);

}  // namespace cilreg
