// 2.5D streaming fourth-order diffusion iteration (diff4th_tiled.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct D4Plan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
};

D4Plan d4_stream_plan(const Dims& d);
// one iteration: reads cur, writes nxt (distinct buffers); isg2 = 1/sigma^2
int d4_stream_step(const D4Plan& T, const float* cur, float* nxt, const float* f, float lam, float tau, float isg2,
                   const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);

}  // namespace cilreg
