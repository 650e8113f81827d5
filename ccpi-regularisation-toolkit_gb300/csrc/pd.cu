// PD-TV: Chambolle-Pock primal-dual TV denoising (reference: PD_TV_core.c:40-252).
//
// One fused kernel per iteration.  State: the extrapolated primal iterate
// Ue (the reference's U after getX) and the dual P, both ping-ponged; the
// kernel recomputes the projected dual at the voxel and at its three lower
// neighbours, so P never makes a second pass through HBM.  Traffic per
// voxel-iteration: read Ue, P(3), f; write Ue, P(3) -> 36 B in 3D.
#include <string.h>

#include "drivers.cuh"
#include "pd_tiled.cuh"

#include <stdlib.h>
#include "nvtx.cuh"

namespace cilreg {

namespace {

struct PdArgs {
    const float* u;      // Ue, current
    float* un;           // Ue, next
    const float* p[3];   // P, current
    float* pn[3];        // P, next
    const float* f;
    float* ubrk;         // U before extrapolation, written on check iterations
    float sigma, tau, lt, theta;
    DoubleDivisor onelt;  // the reference's double (1.0 + lt)
    int nonneg, aniso, check;
};

// projected dual at (i,j,k): P += sigma * mirrored forward difference of Ue
// (PD_TV_core.c:212-229), then the projection of utils.c:180-213
template <bool THREE>
__device__ __forceinline__ void dual_at(const PdArgs& a, const Dims& d, int i, int j, int k, float& p1, float& p2,
                                        float& p3) {
    const long long v = vid(d, i, j, k);
    const float u = ldg(a.u, v);
    p1 = pd_dual(ldg(a.p[0], v), a.sigma, ldg(a.u, vid(d, nb_hi(i, d.nx), j, k)), u);
    p2 = pd_dual(ldg(a.p[1], v), a.sigma, ldg(a.u, vid(d, i, nb_hi(j, d.ny), k)), u);
    p3 = 0.0f;
    if (THREE) p3 = pd_dual(ldg(a.p[2], v), a.sigma, ldg(a.u, vid(d, i, j, nb_hi(k, d.nz))), u);
    if (!a.aniso) {
        pd_project_iso<THREE>(p1, p2, p3);
    } else {
        p1 = pd_project_aniso(p1);
        p2 = pd_project_aniso(p2);
        p3 = pd_project_aniso(p3);
    }
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_pd_step(PdArgs a, Dims d, int kz, const StopCtl* ctl, double2* partials) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    float pa = 0.0f, pb = 0.0f;
    if (i < d.nx && j < d.ny) {
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            float p1, p2, p3, q1, q2, q3, t1, t2, t3;
            dual_at<THREE>(a, d, i, j, k, p1, p2, p3);
            // backward divergence with P[-1] = 0 (PD_TV_core.c:232-252)
            if (i == 0) q1 = -p1;
            else { dual_at<THREE>(a, d, i - 1, j, k, t1, t2, t3); q1 = -(p1 - t1); }
            if (j == 0) q2 = -p2;
            else { dual_at<THREE>(a, d, i, j - 1, k, t1, t2, t3); q2 = -(p2 - t2); }
            float dv = q1 + q2;
            if (THREE) {
                if (k == 0) q3 = -p3;
                else { dual_at<THREE>(a, d, i, j, k - 1, t1, t2, t3); q3 = -(p3 - t3); }
                dv = dv + q3;
            }
            float uo = ldg(a.u, v);
            if (a.nonneg && uo < 0.0f) uo = 0.0f;  // clamp after the dual step (:120)
            const float unew = pd_primal(uo, a.tau, dv, a.lt, ldg(a.f, v), a.onelt);
            if (a.check) {
                const float df = unew - uo;
                pa += df * df;
                pb += unew * unew;
                a.ubrk[v] = unew;
            }
            a.un[v] = pd_extrapolate(unew, a.theta, uo);  // getX (:197-205)
            a.pn[0][v] = p1;
            a.pn[1][v] = p2;
            if (THREE) a.pn[2][v] = p3;
        }
    }
    if (a.check) block_pair_partial<256>(pa, pb, partials, block_slot());
}

// final output: U at the break iteration (already in dst) when stopped,
// otherwise the extrapolated iterate of the last iteration
__global__ void k_pd_select(const StopCtl* ctl, int iter_total, const float* b0, const float* b1, float* dst,
                            long long n) {
    if (ctl->stop) return;
    const float* src = (iter_total & 1) ? b1 : b0;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) dst[i] = src[i];
}

}  // namespace

int pd_run(const float* f, float* u_out, float lam, int iters, float epsil, float lipschitz, int methodTV,
           int nonneg, const Dims& d, cudaStream_t s, float* info) {
    CILREG_RANGE("cilreg PD-TV");
    const bool three = d.nz > 1;
    const int nc = three ? 3 : 2;
    Scratch scratch(s);
    const Launch3 L = plan_launch(d);
    // CILREG_PD_KERNEL=simple selects the per-voxel kernel (kept for A/B checks)
    const char* ek = getenv("CILREG_PD_KERNEL");
    const bool stream = !(ek && strcmp(ek, "simple") == 0);
    const PdPlan T = pd_stream_plan(d);
    const long long nparts = stream ? T.nblocks : num_blocks(L);
    IterControl ctl(s, scratch, iters, epsil, nparts);
    CILREG_TRY(ctl.status());
    float* ub[2];
    float* pb[2][3] = {};
    for (int b = 0; b < 2; b++) {
        ub[b] = scratch.floats(d.n);
        if (!ub[b]) return scratch.status();
        for (int c = 0; c < nc; c++) {
            pb[b][c] = scratch.floats(d.n);
            if (!pb[b][c]) return scratch.status();
        }
    }
    CILREG_CUDA(cudaMemcpyAsync(ub[0], f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    for (int c = 0; c < nc; c++) CILREG_CUDA(cudaMemsetAsync(pb[0][c], 0, sizeof(float) * d.n, s));
    if (iters <= 0) CILREG_CUDA(cudaMemcpyAsync(u_out, f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));

    // step sizes (PD_TV_core.c:50-53): sigma = 1/(L tau) formed in double
    const float tau = lam * 0.1f;
    const float sigma = (float)(1.0 / (double)(lipschitz * tau));
    const float lt = tau / lam;
    const DoubleDivisor onelt = make_double_divisor(1.0 + (double)lt);  // the reference divides by (1.0 + lt)
    int it = 0;
    if (stream && !ctl.checking() && d.n <= (1LL << 22)) {
        // small volume, fixed count: launch overhead dominates, replay a graph
        CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
            PdStreamArgs b;
            b.u = ub[k & 1];
            b.un = ub[(k + 1) & 1];
            for (int c = 0; c < 3; c++) {
                b.p[c] = pb[k & 1][c];
                b.pn[c] = pb[(k + 1) & 1][c];
            }
            b.f = f;
            b.ubrk = u_out;
            b.sigma = sigma;
            b.tau = tau;
            b.lt = lt;
            b.onelt = onelt;
            b.theta = 1.0f;
            b.nonneg = (nonneg == 1);
            b.aniso = (methodTV != 0);
            b.check = 0;
            CILREG_TRY(pd_stream_step(T, b, d, ctl.ctl(), ctl.partials(), st));
            note_launch();
            return OK;
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        PdArgs a;
        a.u = ub[it & 1];
        a.un = ub[(it + 1) & 1];
        for (int c = 0; c < 3; c++) {
            a.p[c] = pb[it & 1][c];
            a.pn[c] = pb[(it + 1) & 1][c];
        }
        a.f = f;
        a.ubrk = u_out;
        a.sigma = sigma;
        a.tau = tau;
        a.lt = lt;
        a.onelt = onelt;
        a.theta = 1.0f;
        a.nonneg = (nonneg == 1);
        a.aniso = (methodTV != 0);
        a.check = check;
        if (stream) {
            PdStreamArgs b;
            b.u = a.u;
            b.un = a.un;
            for (int c = 0; c < 3; c++) {
                b.p[c] = a.p[c];
                b.pn[c] = a.pn[c];
            }
            b.f = f;
            b.ubrk = u_out;
            b.sigma = sigma;
            b.tau = tau;
            b.lt = lt;
            b.onelt = onelt;
            b.theta = 1.0f;
            b.nonneg = a.nonneg;
            b.aniso = a.aniso;
            b.check = check;
            CILREG_TRY(pd_stream_step(T, b, d, ctl.ctl(), ctl.partials(), s));
        } else if (three) {
            k_pd_step<true><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
        } else {
            k_pd_step<false><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
        }
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        if (check) {
            CILREG_TRY(ctl.after_check(it, nparts));
            if (ctl.host_should_stop()) break;
        }
    }
    if (iters > 0) {
        k_pd_select<<<1216, 256, 0, s>>>(ctl.ctl(), iters, ub[0], ub[1], u_out, d.n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
    }
    return ctl.finish(info);
}

}  // namespace cilreg
