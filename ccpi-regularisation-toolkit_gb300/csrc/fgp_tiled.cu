// Shared-memory tiled FGP-TV iteration for 3D volumes (placeholder plan: the
// per-voxel kernel in fgp.cu is used until the tiled kernel is enabled).
#include "fgp_tiled.cuh"

namespace cilreg {

TiledPlan fgp_tiled_plan(const Dims& d) {
    (void)d;
    TiledPlan T;
    T.use = false;
    return T;
}

int fgp_tiled_step(const TiledPlan&, const float* const*, const float* const*, float* const*, const float*, float*,
                   float, float, float, int, int, int, int, int, const Dims&, const StopCtl*, double2*, cudaStream_t) {
    return ERR_ARG;
}

}  // namespace cilreg
