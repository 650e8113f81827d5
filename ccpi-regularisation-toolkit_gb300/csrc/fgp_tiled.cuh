// Shared-memory tiled FGP-TV iteration (3D), see fgp_tiled.cu.
#pragma once

#include "runtime.cuh"

namespace cilreg {

struct TiledPlan {
    bool use = false;
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
    bool x2 = false;  // the two-voxels-per-thread kernel (fgp_x2.cu)
};

// z chunks balanced for `resident_ctas_per_sm` CTAs per SM (0: those of k_fgp_stream)
TiledPlan fgp_tiled_plan(const Dims& d, int resident_ctas_per_sm = 0);
int fgp_default_zchunk(const Dims& d);

// one FGP iteration; with `b` (three device arrays, the unit gradient field
// of a reference image) one FGP-dTV iteration instead; with `carr` the
// momentum coefficient is read on the device as carr[*cbase + coff] (c is
// then unused), so a captured iteration can be replayed at other indices
int fgp_tiled_step(const TiledPlan& T, const float* const pc[3], const float* const po[3], float* const pn[3],
                   const float* f, float* u, float lam, float c, float multip, int nonneg, int aniso, int write_u,
                   int write_p, int check, const Dims& d, const StopCtl* ctl, double2* partials, cudaStream_t s,
                   const float* const* b = nullptr, const float* carr = nullptr, const int* cbase = nullptr,
                   int coff = 0);
// *base += by on the device (one thread)
int fgp_advance_base(int* base, int by, cudaStream_t s);

// The iteration with two voxels per thread (fgp_x2.cu): 2D images and 3D
// volumes of 2^21 voxels or more, nx even and fewer than 2^31 voxels
// (CILREG_FGP_KERNEL=stream or simple keep a one-voxel kernel; use is false
// otherwise).  fgp_tiled_step runs it for a plan with x2 set (FGP-dTV: 2D
// images only, with `b` its reference's unit gradient).
TiledPlan fgp_x2_plan(const Dims& d);
int fgp_x2_step(const TiledPlan& T, const float* const pc[3], const float* const po[3], float* const pn[3],
                const float* f, float* u, float lam, float c, float multip, int nonneg, int aniso, int write_u,
                int write_p, int check, const Dims& d, const StopCtl* ctl, double2* partials, cudaStream_t s,
                const float* carr, const int* cbase, int coff, const float* const* b = nullptr);

// Two iterations k, k+1 in one streaming pass (fgp_pair.cu; 3D only).
struct PairPlan {
    bool use = false;  // CILREG_FGP_PAIR=1 turns pairs on
    dim3 grid, block;
    long long nblocks = 0;
    int zchunk = 0;
};
PairPlan fgp_pair_plan(const Dims& d);
// reads P^{k-1} (pc), P^{k-2} (po) and f, writes P^k (pn1) and P^{k+1} (pn2,
// when write_p2) and U^{k+1} (when write_u2); c1, c2: the momentum
// coefficients of iterations k and k+1.  No stopping check.
int fgp_pair_step(const PairPlan& T, const float* const pc[3], const float* const po[3], float* const pn1[3],
                  float* const pn2[3], const float* f, float* u, float lam, float c1, float c2, float multip,
                  int nonneg, int aniso, int write_u2, int write_p2, const Dims& d, const StopCtl* ctl,
                  cudaStream_t s);

// The iteration with tensor-copy (TMA) staging of its inputs (fgp_tma.cu):
// 3D, x extent a multiple of 4, below 2^31 voxels; CILREG_FGP_TMA=0 turns it off.
bool fgp_tma_usable(const Dims& d);
// tensor maps of the seven staged inputs (pc[0..2], po[0..2], f) into `maps_out`
// (fgp_tma_maps_bytes() bytes); false when an array is not 16-byte aligned or
// the driver refuses the map
bool fgp_tma_encode(const float* const arrays[7], const Dims& d, void* maps_out);
size_t fgp_tma_maps_bytes();
// CTAs of the tensor-copy kernel resident per SM
int fgp_tma_resident();
// same contract as fgp_tiled_step, inputs given by the tensor maps
int fgp_tma_step(const TiledPlan& T, const void* maps, float* const pn[3], float* u, float lam, float c,
                 float multip, int nonneg, int aniso, int write_u, int write_p, int check, const Dims& d,
                 const StopCtl* ctl, double2* partials, cudaStream_t s);
// after a run: fails if a tensor-copy wait timed out (synchronises `s`)
int fgp_tma_status(cudaStream_t s);

// One volume of a batched FGP run (device-resident descriptor table).
struct FgpBatchVol {
    Dims d;
    const float* f;
    float* u;
    float* ring[3][3];   // three P buffers x three components
    StopCtl* ctl;
    double2* partials;   // this volume's slots, one per tile
    float lam, multip;
    long long tile_base; // first flat tile index of this volume
    int gx, gy, gz, zc;  // tile grid and z chunk of this volume
};

// Persistent batched run (one launch for every iteration of every volume):
// the device-side work queue and dependency counters of k_fgp_persistent.
struct FgpPersistArgs {
    const FgpBatchVol* vols;
    const int* tile_vol;
    const float* carr;          // momentum coefficient of each iteration
    unsigned long long* next;   // work-item counter (zero before the launch)
    unsigned long long* arrive; // per volume: tiles finished since it0
    int* release;               // per volume: iterations released (it0 before the launch)
    int* error;                 // set when a dependency wait ran out
    const long long* gtile;     // group g holds flat tiles [gtile[g], gtile[g+1])
    const long long* gitem;     // group g's first work item; gitem[ngroups] = all items
    int ngroups;
    int it0, iters;             // iterations it0 .. it0 + (items of a group) / (its tiles) - 1 of `iters`
    int nonneg, aniso, checking;
    float epsil;
    long long wait_limit;       // polls (about 0.2 us each) before a wait gives up
};
int fgp_persistent_launch(const FgpPersistArgs& A, bool three, bool wide, int nctas, cudaStream_t s);
// CTAs of the persistent kernel resident on the device at once
int fgp_persistent_ctas();

// tile grid of one volume for the streaming kernel with z chunk `zc`
void fgp_tile_grid(const Dims& d, int zc, int& gx, int& gy, int& gz);

// one iteration `it` of every volume: flat grid over all tiles, tile_vol maps
// a flat tile to its volume; all volumes share dimensionality `three`; `wide`
// when some volume has 2^31 voxels or more (64-bit element offsets)
int fgp_batch_step(const FgpBatchVol* d_vols, const int* d_tile_vol, long long ntiles, bool three, bool wide, int it,
                   float c, int nonneg, int aniso, int write_u, int write_p, int check, cudaStream_t s);

// the same with the two-voxel tile (fgp_x2.cu; the 2D tile for volumes of one
// plane): every volume with nx even, below 2^31 voxels, f and u 8-byte
// aligned; its tile grid per volume
bool fgp_x2_batch_usable(const Dims* dims, const float* const* f, float* const* u, int nvol);
void fgp_x2_tile_grid(const Dims& d, int zc, int& gx, int& gy, int& gz);
int fgp_x2_batch_step(const FgpBatchVol* d_vols, const int* d_tile_vol, long long ntiles, int it, float c,
                      int nonneg, int aniso, int write_u, int write_p, int check, cudaStream_t s);

}  // namespace cilreg
