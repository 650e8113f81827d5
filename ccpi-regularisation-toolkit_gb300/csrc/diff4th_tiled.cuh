// 2.5D streaming fourth-order diffusion iteration (diff4th_tiled.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct D4Plan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool pair = false;  // the two-voxels-per-thread kernel (diff4th_pair.cu)
};

// the plan of the streaming kernel that runs for `d`: volumes with nx even
// and fewer than 2^31 voxels run k_d4_pair (3D) or k_d4_pair2d
// (CILREG_D4_KERNEL=stream selects k_d4_stream), others k_d4_stream
D4Plan d4_stream_plan(const Dims& d);
bool d4_pair_applies(const Dims& d);
D4Plan d4_pair_plan(const Dims& d);
int d4_pair_step(const D4Plan& T, const float* cur, float* nxt, const float* f, float lam, float tau, float isg2,
                 const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);
// one iteration: reads cur, writes nxt (distinct buffers); isg2 = 1/sigma^2
int d4_stream_step(const D4Plan& T, const float* cur, float* nxt, const float* f, float lam, float tau, float isg2,
                   const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);

}  // namespace cilreg
