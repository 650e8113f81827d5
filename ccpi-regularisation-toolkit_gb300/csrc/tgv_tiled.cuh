// TGV dual and primal half-iterations as 2.5D streaming kernels (tgv_tiled.cu).
#pragma once

#include "tgv_batch.cuh"

namespace cilreg {

struct TgvPlan {
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool use = false;  // false: the per-voxel kernels of tgv.cu run instead
    bool tma = false;  // fused pass: inputs staged by tensor copies (tgv_fused_tma.cu)
};

TgvPlan tgv_primal_plan(const Dims& d);
int tgv_primal_stream_step(const TgvPlan& T, const TgvArgs& a, const Dims& d, const StopCtl* ctl, double2* partials,
                           cudaStream_t s);

// the dual half-iteration as a streaming kernel on the same tiling (forward
// differences: a one-voxel halo on the high x/y sides), single volume / batch
int tgv_dual_stream_step(const TgvPlan& T, const TgvArgs& a, const Dims& d, const StopCtl* ctl, cudaStream_t s);
int tgv_dual_batch_step(const TgvBatchVol* d_vols, const int* d_ptile_vol, long long nptiles, bool three,
                        cudaStream_t s);

// one whole iteration (dual and primal halves) in one pass over double-
// buffered state (tgv_fused.cu; 3D, below 2^31 voxels; CILREG_TGV_FUSED=0
// turns it off)
struct TgvFusedArgs {
    const float* u;   // extrapolated U (old)
    const float* u0;
    const float* v[3];
    const float* p[3];
    const float* q[6];
    float* un;        // new
    float* vn[3];
    float* pn[3];
    float* qn[6];
    float lambda, alpha1, alpha0, tau, sigma, inv_lt;
};
TgvPlan tgv_fused_plan(const Dims& d);

// one volume of a batched run of the fused pass (device descriptor table)
struct TgvFusedVol {
    Dims d;
    TgvFusedArgs args[2];  // iteration parity 0: buffers 0 -> 1, parity 1: 1 -> 0
    StopCtl* ctl;
    double2* partials;     // one slot per tile of this volume
    long long tile_base;   // first flat tile index of this volume
    int gx, gy, gz, zc;
};
// tiling of the fused pass in a batched run (64-plane chunks)
void tgv_fused_tiles(const Dims& d, int& gx, int& gy, int& gz, int& zc);
int tgv_fused_batch_step(const TgvFusedVol* d_vols, const int* d_tile_vol, long long ntiles, int parity, int check,
                         cudaStream_t s);
int tgv_fused_step(const TgvPlan& T, const TgvFusedArgs& a, const Dims& d, const StopCtl* ctl, int check,
                   double2* partials, cudaStream_t s);

// the fused pass with its 14 input arrays staged by tensor copies
// (tgv_fused_tma.cu): 3D volumes whose x extent is a multiple of 4 and whose
// arrays start on 16-byte boundaries; CILREG_TGV_TMA=0 turns it off
bool tgv_tma_usable(const Dims& d);
int tgv_tma_resident();  // CTAs per SM of the staged kernel (0 if it cannot run)
size_t tgv_tma_maps_bytes();
// tensor maps of a's input arrays into maps_out (tgv_tma_maps_bytes() bytes);
// false if an array is not 16-byte aligned or the driver refuses a map
bool tgv_tma_encode(const TgvFusedArgs& a, const Dims& d, void* maps_out);
int tgv_tma_step(const TgvPlan& T, const void* maps, const TgvFusedArgs& a, const Dims& d, const StopCtl* ctl,
                 int check, double2* partials, cudaStream_t s);
// fails if a tensor-copy wait of the staged kernel ran out (and clears the flag)
int tgv_tma_status(cudaStream_t s);
// batched runs of the staged pass: every volume qualifies (x extent a
// multiple of 4, below 2^31 voxels); d_maps holds, for volume v and parity
// p, the maps of args[p]'s input arrays at d_maps + (2 v + p) x
// tgv_tma_maps_bytes()
bool tgv_tma_batch_usable(const Dims* dims, int nvol);
int tgv_tma_batch_step(const TgvFusedVol* d_vols, const int* d_tile_vol, const void* d_maps, long long ntiles,
                       int parity, int check, cudaStream_t s);

// tiling of the streaming primal kernel in a batched run (64-plane chunks)
void tgv_primal_tiles(const Dims& d, int& gx, int& gy, int& gz, int& zc);
// primal half-iteration of every volume of a batch: one flat grid over the
// volumes' streaming tiles (TgvBatchVol::ptile_base.., tile -> volume map)
int tgv_primal_batch_step(const TgvBatchVol* d_vols, const int* d_ptile_vol, long long nptiles, bool three, int check,
                          cudaStream_t s);

}  // namespace cilreg
