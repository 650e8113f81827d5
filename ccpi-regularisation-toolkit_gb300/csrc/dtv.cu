// FGP-dTV: FGP on the directional total variation of a reference image
// (reference: FGP_dTV_core.c:46-380).
//
// Once per call the eta-smoothed unit gradient field B of the reference image
// is formed (GradNorm_func, FGP_dTV_core.c:273-300).  Each iteration then is
// the FGP iteration with R and the gradient of U projected onto the
// orthogonal complement of B at every voxel; it runs on the FGP streaming
// kernel's dTV variant (fgp_tiled.cu): one launch per iteration reading
// P^{k-1}, P^{k-2}, f and B and writing P^k (52 B per voxel in 3D), R and U
// never stored.  The momentum recurrence and the stopping rule are FGP's;
// t_{k+1} is formed with a double square root as the reference does.
#include <math.h>

#include <vector>

#include "drivers.cuh"
#include "fgp_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

// B = grad(ref) / sqrt(|grad(ref)|^2 + eta^2), forward differences with the
// reference value 0 beyond the last index (FGP_dTV_core.c:187-205, 273-300)
template <bool THREE>
__global__ void __launch_bounds__(256) k_dtv_gradnorm(const float* __restrict__ ref, float* __restrict__ bx,
                                                      float* __restrict__ by, float* __restrict__ bz, float eta_sq,
                                                      Dims d, int kz) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    if (i >= d.nx || j >= d.ny) return;
    for (int kk = 0; kk < kz; kk++) {
        const int k = k0 + kk;
        if (k >= d.nz) break;
        const long long v = (long long)k * d.sxy + (long long)j * d.nx + i;
        const float b = __ldg(ref + v);
        const float gx = ((i == d.nx - 1) ? 0.0f : __ldg(ref + v + 1)) - b;
        const float gy = ((j == d.ny - 1) ? 0.0f : __ldg(ref + v + d.nx)) - b;
        float m = __fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy));
        float gz = 0.0f;
        if (THREE) {
            gz = ((k == d.nz - 1) ? 0.0f : __ldg(ref + v + d.sxy)) - b;
            m = __fadd_rn(m, __fmul_rn(gz, gz));
        }
        // the reference's double square root of a float, rounded to float,
        // equals the correctly rounded single-precision square root
        const float magn = sqrtf(__fadd_rn(m, eta_sq));
        bx[v] = __fdiv_rn(gx, magn);
        by[v] = __fdiv_rn(gy, magn);
        if (THREE) bz[v] = __fdiv_rn(gz, magn);
    }
}

}  // namespace

int dtv_run(const float* f, const float* ref, float* u_out, float lam, int iters, float epsil, float eta,
            int methodTV, int nonneg, const Dims& d, cudaStream_t s, float* info) {
    CILREG_RANGE("cilreg FGP-dTV");
    if (!ref) return fail(ERR_ARG, __FILE__, __LINE__, "null reference image");
    const bool three = d.nz > 1;
    const int nc = three ? 3 : 2;
    Scratch scratch(s);
    // 2D images with an even row length: the two-pixel kernel; otherwise the
    // streaming kernel (whatever CILREG_FGP_KERNEL says, bar 'stream')
    TiledPlan T = fgp_tiled_plan(d);
    if (d.nz == 1) {
        const TiledPlan X = fgp_x2_plan(d);
        if (X.use) T = X;
    }
    IterControl ctl(s, scratch, iters, epsil, T.nblocks);
    CILREG_TRY(ctl.status());
    float* ring[3][3] = {};
    float* b[3] = {nullptr, nullptr, nullptr};
    for (int c = 0; c < nc; c++) {
        b[c] = scratch.floats(d.n);
        if (!b[c]) return scratch.status();
        for (int r = 0; r < 3; r++) {
            ring[r][c] = scratch.floats(d.n);
            if (!ring[r][c]) return scratch.status();
        }
    }
    // P^{-1} = P^{-2} = 0 (calloc'd P, P_prev, R of the reference)
    for (int r = 1; r < 3; r++)
        for (int c = 0; c < nc; c++) CILREG_CUDA(cudaMemsetAsync(ring[r][c], 0, sizeof(float) * d.n, s));
    {
        const Launch3 L = plan_launch(d);
        const float eta_sq = eta * eta;
        if (three)
            k_dtv_gradnorm<true><<<L.grid, L.block, 0, s>>>(ref, b[0], b[1], b[2], eta_sq, d, L.kz);
        else
            k_dtv_gradnorm<false><<<L.grid, L.block, 0, s>>>(ref, b[0], b[1], nullptr, eta_sq, d, L.kz);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
    }
    const float multip = three ? (1.0f / (26.0f * lam)) : (1.0f / (8.0f * lam));  // FGP_dTV_core.c:240, 338
    float tk = 1.0f, cprev = 0.0f;
    // t_{k+1} = (1 + sqrt(1 + 4 t_k^2)) / 2 in double, as FGP_dTV_core.c:144
    auto advance = [&]() {
        const float tkp1 = (float)((1.0f + sqrt((double)(1.0f + 4.0f * tk * tk))) * 0.5f);
        cprev = (tk - 1.0f) / tkp1;
        tk = tkp1;
    };
    int it = 0;
    constexpr int G = 66;  // replayed block: a multiple of the ring's period 3
    if (!ctl.checking() && d.n <= (1LL << 22) && iters > 2 * G) {
        // small image or volume, fixed count: iterations 0 .. iters-2 from a
        // replayed graph, their momentum coefficients read on the device from
        // the sequence formed here; the last one (U written, no P) directly
        std::vector<float> cseq(iters);
        for (int k = 0; k < iters; k++) {
            cseq[k] = cprev;
            advance();
        }
        float* carr = scratch.floats(iters);
        int* cbase = (int*)scratch.bytes(sizeof(int));
        if (!carr || !cbase) return scratch.status();
        CILREG_CUDA(cudaMemcpyAsync(carr, cseq.data(), sizeof(float) * iters, cudaMemcpyHostToDevice, s));
        CILREG_CUDA(cudaMemsetAsync(cbase, 0, sizeof(int), s));
        auto iteration = [&](int k, cudaStream_t st, bool in_graph) -> int {
            float* pn[3] = {ring[k % 3][0], ring[k % 3][1], ring[k % 3][2]};
            const float* pc[3] = {ring[(k + 2) % 3][0], ring[(k + 2) % 3][1], ring[(k + 2) % 3][2]};
            const float* po[3] = {ring[(k + 1) % 3][0], ring[(k + 1) % 3][1], ring[(k + 1) % 3][2]};
            const int last = (k == iters - 1) ? 1 : 0;
            CILREG_TRY(fgp_tiled_step(T, pc, po, pn, f, u_out, lam, cseq[k], multip, nonneg == 1, methodTV != 0, last,
                                      1 - last, 0, d, ctl.ctl(), ctl.partials(), st, b, in_graph ? carr : nullptr,
                                      cbase, k));
            note_launch();
            return OK;
        };
        CILREG_TRY(run_replayed(iters - 1, G, s, iteration,
                                [&](cudaStream_t st) -> int { return fgp_advance_base(cbase, G, st); }));
        CILREG_TRY(iteration(iters - 1, s, false));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        float* pn[3];
        const float* pc[3];
        const float* po[3];
        for (int c = 0; c < 3; c++) {
            pn[c] = ring[it % 3][c];
            pc[c] = ring[(it + 2) % 3][c];
            po[c] = ring[(it + 1) % 3][c];
        }
        const int write_u = (it == iters - 1) || check || (ctl.checking() && ((it + 1) % 5 == 0));
        const int write_p = (it != iters - 1);
        CILREG_TRY(fgp_tiled_step(T, pc, po, pn, f, u_out, lam, cprev, multip, nonneg == 1, methodTV != 0, write_u,
                                  write_p, check, d, ctl.ctl(), ctl.partials(), s, b));
        note_launch();
        advance();
        if (check) {
            CILREG_TRY(ctl.after_check(it, T.nblocks));
            if (ctl.host_should_stop()) break;
        }
    }
    return ctl.finish(info);
}

}  // namespace cilreg
