// Shared-memory tiled FGP-TV iteration (3D), see fgp_tiled.cu.
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct TiledPlan {
    bool use = false;
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
};

TiledPlan fgp_tiled_plan(const Dims& d);

int fgp_tiled_step(const TiledPlan& T, const float* const pc[3], const float* const po[3], float* const pn[3],
                   const float* f, float* u, float lam, float c, float multip, int nonneg, int aniso, int write_u,
                   int write_p, int check, const Dims& d, const StopCtl* ctl, double2* partials, cudaStream_t s);

}  // namespace cilreg
