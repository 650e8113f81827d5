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
// tile grid is plan_launch(d): 32 x 8 threads, kz planes per thread.
struct TgvBatchVol {
    Dims d;
    TgvArgs args;
    StopCtl* ctl;
    double2* partials;    // this volume's slots, one per tile
    long long tile_base;  // first flat tile index of this volume
    int gx, gy, gz, kz;
};

// one iteration (dual then primal kernel) of every volume
int tgv_batch_step(const TgvBatchVol* d_vols, const int* d_tile_vol, long long ntiles, bool three, int check,
                   cudaStream_t s);

}  // namespace cilreg
