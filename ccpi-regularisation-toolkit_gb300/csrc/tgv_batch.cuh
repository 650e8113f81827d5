// TGV kernel arguments and the batched-run descriptor (tgv.cu, batch.cu).
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct TgvArgs {
    float* u;
    const float* u0;
    float* p[3];
    float* q[6];
    float* v[3];
    float lambda, alpha1, alpha0, tau, sigma;
    float inv_lt;  // 1 / (lambda + tau)
    int check;
};

// One volume of a batched TGV run (device-resident descriptor table).  The
// dual kernel's tiles are plan_launch(d) (32 x 8 threads, kz planes per
// thread); the streaming primal kernel's are tgv_primal_tiles(d).
struct TgvBatchVol {
    Dims d;
    TgvArgs args;
    StopCtl* ctl;
    double2* partials;     // this volume's stopping-rule slots, one per primal tile
    long long tile_base;   // first flat dual tile index of this volume
    long long ptile_base;  // first flat primal tile index of this volume
    int gx, gy, gz, kz;    // dual tiling
    int pgx, pgy, pgz, pzc;  // primal tiling
};

// one iteration (dual then primal kernel) of every volume
int tgv_batch_step(const TgvBatchVol* d_vols, const int* d_tile_vol, long long ntiles, const int* d_ptile_vol,
                   long long nptiles, bool three, int check, cudaStream_t s);

}  // namespace cilreg
