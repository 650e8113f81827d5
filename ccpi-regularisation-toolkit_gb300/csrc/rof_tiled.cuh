// 2.5D streaming ROF-TV iteration (rof_tiled.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct RofPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool pair = false;  // the two-voxels-per-thread kernel (rof_pair.cu)
};

RofPlan rof_tiled_plan(const Dims& d);

// volumes and images with nx even and fewer than 2^31 voxels run k_rof_pair
// (3D) or k_rof_pair2d (CILREG_ROF_KERNEL=async, reg or simple select a
// one-voxel kernel)
bool rof_pair_applies(const Dims& d);
RofPlan rof_pair_plan(const Dims& d);
int rof_pair_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                  float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);

// one iteration: reads cur, writes nxt; on a check iteration one FP64 partial
// per CTA (RofPlan::nblocks of them)
int rof_tiled_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                   float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);

// 2D images, fixed counts: iterations per launch of the overlapped-halo
// kernel, CILREG_ROF_TB=<depth> (at most 8); 0 (the default) when it is not
// asked for or does not apply
int rof_tb2d_depth(const Dims& d, int iters);
// `depth` iterations in one launch: reads cur, writes nxt (distinct buffers)
int rof_tb2d_step(const float* cur, float* nxt, const float* f, const float* lam_arr, float lam, float tau,
                  const Dims& d, int depth, cudaStream_t s);

// 2D images at a fixed count: all iterations in one cooperative launch of
// k_rof_persist2d (rof_persist.cu) when every 32 x 64 tile can be resident at
// once; opt-in, CILREG_ROF_PERSIST=1 (slower than graph-replayed launches)
bool rof_persist2d_applies(const Dims& d, int iters);
long long rof_persist2d_tiles(const Dims& d);
// U^0 in g0; U^iters ends in g[iters & 1]; flags: one int per tile, error one
// int (set when a wait between tiles ran out)
int rof_persist2d_run(float* g0, float* g1, const float* f, const float* lam_arr, float lam, float tau, int iters,
                      const Dims& d, int* flags, int* error, cudaStream_t s);

}  // namespace cilreg
