// 2.5D streaming PD-TV iteration (pd_tiled.cu).
#pragma once

#include "pd_math.cuh"
#include "runtime.cuh"

namespace cilreg {

struct PdStreamArgs {
    const float* u;     // extrapolated primal iterate Ue (current)
    float* un;          // Ue (next)
    const float* p[3];  // dual (current)
    float* pn[3];       // dual (next)
    const float* f;
    float* ubrk;        // U before extrapolation, written on check iterations
    float sigma, tau, lt, theta;
    DoubleDivisor onelt;  // the reference's double (1.0 + lt)
    int nonneg, aniso, check;
};

struct PdPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
};

PdPlan pd_stream_plan(const Dims& d);
int pd_stream_step(const PdPlan& T, const PdStreamArgs& a, const Dims& d, const StopCtl* ctl, double2* partials,
                   cudaStream_t s);

}  // namespace cilreg
