// Device-pointer drivers, one per regulariser.  Every driver:
//   * takes device pointers and the stream all of its work is enqueued on;
//   * allocates its state from the stream-ordered pool and frees it on return;
//   * runs the whole iteration loop without a per-iteration host sync (the
//     stopping rule is evaluated on the device, see common.cuh);
//   * writes infovector = [iterations run, last relative change] to the host
//     pointer `info` (may be null) and returns 0 or a negative Status.
// The argument meanings are those of the reference's *_CPU_main functions
// (src/Core/regularisers_CPU/*_core.h), with dims as a Dims value.
#pragma once

#include "runtime.cuh"

namespace cilreg {

// Device state a regulariser keeps between calls (warm start across the outer
// iterations of a proximal-splitting solver).  Owned by the caller.
struct FgpWarm {
    float* ring[3][3];  // the three dual buffers (P_{k-1}, P_{k-2}, P_k)
    int base;           // ring index offset: iteration it writes ring[(base + it) % 3]
};
struct SbWarm {
    float* dd[3];  // D (split variable)
    float* bb[3];  // B (Bregman variable)
};

// ROF_TV_core.c:50-99.  lam_arr (device, per voxel) overrides lam when non-null.
// u_init (device, optional) replaces f as the starting iterate
int rof_run(const float* f, float* u_out, const float* lam_arr, float lam, int iters, float tau, float epsil,
            const Dims& d, cudaStream_t s, float* info, const float* u_init = nullptr);

// One ROF iteration (the kernel rof_run launches) on caller-provided buffers:
// reads `cur`, writes `nxt`; on a check iteration writes one FP64 partial per
// CTA (num_blocks(plan_launch(d)) of them) for launch_finalize_check.
int rof_launch_step(const float* cur, float* nxt, const float* f, const float* lam_arr, float lam, float tau,
                    const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s);
// number of FP64 partial slots rof_launch_step writes on a check iteration
long long rof_partial_slots(const Dims& d);
// OK when the kernel rof_launch_step would run for `d` fits the launch grid
// limits, else an argument error naming the shape
int rof_check_grid(const Dims& d);

// FGP_TV_core.c:40-171.  u_out's initial content is U_prev of iteration 0.
// warm (optional): dual state carried across calls; its ring is updated
int fgp_run(const float* f, float* u_out, float lam, int iters, float epsil, int methodTV, int nonneg,
            const Dims& d, cudaStream_t s, float* info, FgpWarm* warm = nullptr);

// PD_TV_core.c:40-153
int pd_run(const float* f, float* u_out, float lam, int iters, float epsil, float lipschitz, int methodTV,
           int nonneg, const Dims& d, cudaStream_t s, float* info);

// SB_TV_core.c:38-144
// warm (optional): D and B carried across calls
int sb_run(const float* f, float* u_out, float mu, int iters, float epsil, int methodTV, const Dims& d,
           cudaStream_t s, float* info, SbWarm* warm = nullptr);

// TGV_core.c:43-194
int tgv_run(const float* f, float* u_out, float lam, float alpha1, float alpha0, int iters, float L2, float epsil,
            const Dims& d, cudaStream_t s, float* info);

// Diffusion_core.c:53-102, Jacobi update order
// u_init (device, optional) replaces f as the starting iterate
int ndf_run(const float* f, float* u_out, float lam, float sigma, int iters, float tau, int penalty, float epsil,
            const Dims& d, cudaStream_t s, float* info, const float* u_init = nullptr);

// Diffus4th_order_core.c:44-99
int diff4th_run(const float* f, float* u_out, float lam, float sigma, int iters, float tau, float epsil,
                const Dims& d, cudaStream_t s, float* info);

// FGP_dTV_core.c:46-180.  ref: the reference image (device); u_out's initial
// content is U_prev of iteration 0, as for FGP
int dtv_run(const float* f, const float* ref, float* u_out, float lam, int iters, float epsil, float eta,
            int methodTV, int nonneg, const Dims& d, cudaStream_t s, float* info);

// LLT_ROF_core.c:54-117
int llt_run(const float* f, float* u_out, float lam_rof, float lam_llt, int iters, float tau, float epsil,
            const Dims& d, cudaStream_t s, float* info);

// shape validation shared by every entry point
int check_dims(int nx, int ny, int nz);

}  // namespace cilreg
