// Linear and non-linear diffusion, explicit scheme (reference:
// Diffusion_core.c:53-413), Jacobi update order.
//
// The reference's C-OMP sweep updates U in place, so a voxel reads
// neighbours that other threads may or may not have updated already (the
// result depends on the thread count).  Here every sweep reads the previous
// iterate only (ping-pong buffers): deterministic, and equal to the
// reference run with one thread up to the update order.  One kernel per
// iteration: a 2.5D streaming kernel (12 B of HBM traffic per
// voxel-iteration; two voxels per thread in ndf_pair.cu for 3D volumes with
// an even row length, one in ndf_tiled.cu otherwise), or the per-voxel kernel
// below for CILREG_NDF_KERNEL=simple and volumes of 2^31 voxels or more.
#include "drivers.cuh"
#include "ndf_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {

namespace {

template <bool THREE, int PEN>
__global__ void __launch_bounds__(256) k_ndf_step(const float* __restrict__ U, float* __restrict__ Un,
                                                  const float* __restrict__ F, float lam, float sg, float isg, float tau,
                                                  Dims d, int kz, const StopCtl* ctl, int check, double2* partials) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    float pa = 0.0f, pb = 0.0f;
    if (i < d.nx && j < d.ny) {
        const int il = nb_lo(i, d.nx), ih = nb_hi(i, d.nx), jl = nb_lo(j, d.ny), jh = nb_hi(j, d.ny);
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            const float c = ldg(U, v);
            const float e1 = flux<PEN>(ldg(U, vid(d, ih, j, k)) - c, sg, isg);
            const float w1 = flux<PEN>(ldg(U, vid(d, il, j, k)) - c, sg, isg);
            const float n1 = flux<PEN>(ldg(U, vid(d, i, jh, k)) - c, sg, isg);
            const float s1 = flux<PEN>(ldg(U, vid(d, i, jl, k)) - c, sg, isg);
            float sum;
            if (THREE) {
                const float u1 = flux<PEN>(ldg(U, vid(d, i, j, nb_hi(k, d.nz))) - c, sg, isg);
                const float d1 = flux<PEN>(ldg(U, vid(d, i, j, nb_lo(k, d.nz))) - c, sg, isg);
                sum = e1 + w1 + n1 + s1 + u1 + d1;
            } else {
                sum = e1 + w1 + n1 + s1;
            }
            const float un = c + tau * (lam * sum - (c - ldg(F, v)));
            Un[v] = un;
            if (check) {
                const float df = un - c;
                pa += df * df;
                pb += un * un;
            }
        }
    }
    if (check) block_pair_partial<256>(pa, pb, partials, block_slot());
}

template <bool THREE>
void launch_ndf(int pen, const Launch3& L, cudaStream_t s, const float* U, float* Un, const float* F, float lam,
                float sg, float isg, float tau, const Dims& d, const StopCtl* ctl, int check, double2* part) {
#define NDF_CASE(P)                                                                                       \
    case P:                                                                                               \
        k_ndf_step<THREE, P><<<L.grid, L.block, 0, s>>>(U, Un, F, lam, sg, isg, tau, d, L.kz, ctl, check, part); \
        break;
    switch (pen) {
        NDF_CASE(0)
        NDF_CASE(1)
        NDF_CASE(2)
        NDF_CASE(3)
        NDF_CASE(4)
        NDF_CASE(5)
        default: break;
    }
#undef NDF_CASE
}

}  // namespace

int ndf_run(const float* f, float* u_out, float lam, float sigma, int iters, float tau, int penalty, float epsil,
            const Dims& d, cudaStream_t s, float* info, const float* u_init) {
    CILREG_RANGE("cilreg NDF");
    const bool linear = (sigma == 0.0f);
    if (!linear && (penalty < 1 || penalty > 5))
        return fail(ERR_ARG, __FILE__, __LINE__, "No penalty function selected! Use 1,2,3,4 or 5.");
    const int pen = linear ? 0 : penalty;
    const float sg_ref = (float)((double)sigma / sqrt(2.0));  // Diffusion_core.c:57
    const float isg = linear ? 0.0f : 1.0f / sg_ref;
    // the kernels compare |e| with sg only; below 0 every such comparison
    // gives what it gives at 0 up to the sign of a zero flux, and from 0 on a
    // flux whose sign is taken has e != 0 (flux in ndf_tiled.cuh)
    const float sg = fmaxf(sg_ref, 0.0f);
    const bool three = d.nz > 1;
    Scratch scratch(s);
    const Launch3 L = plan_launch(d);
    const NdfPlan T = ndf_stream_plan(d);
    const long long nparts = T.use ? T.nblocks : num_blocks(L);
    IterControl ctl(s, scratch, iters, epsil, nparts);
    CILREG_TRY(ctl.status());
    float* alt = scratch.floats(d.n);
    if (!alt) return scratch.status();
    float* bufs[2] = {u_out, alt};
    CILREG_CUDA(cudaMemcpyAsync(u_out, u_init ? u_init : f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    int it = 0;
    if (!ctl.checking() && d.n <= (1LL << 22)) {
        // small volume, fixed count: launch overhead dominates, replay a graph
        CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
            if (T.use)
                CILREG_TRY(ndf_stream_step(T, pen, bufs[k & 1], bufs[(k + 1) & 1], f, lam, sg, isg, tau, d,
                                           ctl.ctl(), 0, ctl.partials(), st));
            else if (three)
                launch_ndf<true>(pen, L, st, bufs[k & 1], bufs[(k + 1) & 1], f, lam, sg, isg, tau, d, ctl.ctl(), 0,
                                 ctl.partials());
            else
                launch_ndf<false>(pen, L, st, bufs[k & 1], bufs[(k + 1) & 1], f, lam, sg, isg, tau, d, ctl.ctl(), 0,
                                  ctl.partials());
            CILREG_CUDA(cudaGetLastError());
            note_launch();
            return OK;
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        if (T.use)
            CILREG_TRY(ndf_stream_step(T, pen, bufs[it & 1], bufs[(it + 1) & 1], f, lam, sg, isg, tau, d, ctl.ctl(),
                                       check, ctl.partials(), s));
        else if (three)
            launch_ndf<true>(pen, L, s, bufs[it & 1], bufs[(it + 1) & 1], f, lam, sg, isg, tau, d, ctl.ctl(), check,
                             ctl.partials());
        else
            launch_ndf<false>(pen, L, s, bufs[it & 1], bufs[(it + 1) & 1], f, lam, sg, isg, tau, d, ctl.ctl(), check,
                              ctl.partials());
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        if (check) {
            CILREG_TRY(ctl.after_check(it, nparts));
            if (ctl.host_should_stop()) break;
        }
    }
    if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl.ctl(), iters, bufs, u_out, d.n, s));
    return ctl.finish(info);
}

}  // namespace cilreg
