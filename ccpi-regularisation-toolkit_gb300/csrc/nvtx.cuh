// NVTX ranges (the header-only NVTX v3 of the CUDA toolkit): each regulariser
// run, batched run, prox-session loop, adjoint and graph launch is a named
// range on the Nsight timelines.  With no tool attached a range costs one
// check of an unset function pointer.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace cilreg {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace cilreg

#define CILREG_RANGE(name) ::cilreg::NvtxRange cilreg_nvtx_range_(name)
