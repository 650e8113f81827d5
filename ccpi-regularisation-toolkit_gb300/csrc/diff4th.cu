// Fourth-order anisotropic diffusion (Hajiaboli), explicit scheme
// (reference: Diffus4th_order_core.c:44-265).
//
// Two kernels per iteration: the weighted Laplacian W of U (19-point stencil
// in 3D), then U += tau (-lambda Lap(W) - (U - f)) in place (each voxel
// reads W at its mirrored neighbours and U, f at itself only).
#include "diff4th_tiled.cuh"
#include <string.h>

#include "drivers.cuh"

#include <stdlib.h>
#include "nvtx.cuh"

namespace cilreg {

namespace {

template <bool THREE>
__global__ void __launch_bounds__(256) k_d4_laplacian(const float* __restrict__ U, float* __restrict__ W, float isg2,
                                                      Dims d, int kz, const StopCtl* ctl) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    if (i >= d.nx || j >= d.ny) return;
    const int im = nb_lo(i, d.nx), ip = nb_hi(i, d.nx), jm = nb_lo(j, d.ny), jp = nb_hi(j, d.ny);
    const float EPS = 1.0e-7f;
    for (int kk = 0; kk < kz; kk++) {
        const int k = k0 + kk;
        if (k >= d.nz) break;
        const long long v = vid(d, i, j, k);
        const float c0 = ldg(U, v);
        const float xm = ldg(U, vid(d, im, j, k)), xp = ldg(U, vid(d, ip, j, k));
        const float ym = ldg(U, vid(d, i, jm, k)), yp = ldg(U, vid(d, i, jp, k));
        const float gx = 0.5f * (xm - xp), gy = 0.5f * (ym - yp);
        const float gx2 = gx * gx, gy2 = gy * gy;
        const float gxx = xm + xp - 2.0f * c0;
        const float gyy = ym + yp - 2.0f * c0;
        const float gxy = 0.25f * (ldg(U, vid(d, im, jm, k)) + ldg(U, vid(d, ip, jp, k)) - ldg(U, vid(d, im, jp, k)) -
                                   ldg(U, vid(d, ip, jm, k)));
        const float xy2 = 2.0f * gx * gy * gxy;
        float den, vn, vo;
        if (THREE) {
            const int km = nb_lo(k, d.nz), kp = nb_hi(k, d.nz);
            const float zm = ldg(U, vid(d, i, j, km)), zp = ldg(U, vid(d, i, j, kp));
            const float gz = 0.5f * (zm - zp);
            const float gz2 = gz * gz;
            const float gzz = zm + zp - 2.0f * c0;
            // Diffus4th_order_core.c:210-212
            const float gxz = 0.25f * (ldg(U, vid(d, im, j, km)) - ldg(U, vid(d, ip, j, km)) -
                                       ldg(U, vid(d, im, j, kp)) + ldg(U, vid(d, ip, j, kp)));
            const float gyz = 0.25f * (ldg(U, vid(d, i, jm, km)) - ldg(U, vid(d, i, jp, km)) -
                                       ldg(U, vid(d, i, jm, kp)) + ldg(U, vid(d, i, jp, kp)));
            const float xz2 = 2.0f * gx * gz * gxz;
            const float yz2 = 2.0f * gy * gz * gyz;
            den = gx2 + gy2 + gz2;
            const float nn = gxx * gx2 + gyy * gy2 + gzz * gz2 + xy2 + xz2 + yz2;
            const float oo = (gy2 + gz2) * gxx + (gx2 + gz2) * gyy + (gx2 + gy2) * gzz - xy2 - xz2 - yz2;
            const float iq = __frcp_rn((den <= EPS) ? EPS : den);  // one reciprocal for both quotients
            vn = nn * iq;
            vo = oo * iq;
        } else {
            den = gx2 + gy2;
            const float nn = gxx * gx2 + xy2 + gyy * gy2;
            const float oo = gxx * gy2 - xy2 + gyy * gx2;
            const float iq = __frcp_rn((den <= EPS) ? EPS : den);
            vn = nn * iq;
            vo = oo * iq;
        }
        const float c = __frcp_rn(1.0f + den * isg2);
        W[v] = (c * c) * vn + c * vo;
    }
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_d4_update(float* __restrict__ U, const float* __restrict__ W,
                                                   const float* __restrict__ F, float lam, float tau, Dims d, int kz,
                                                   const StopCtl* ctl, int check, double2* partials) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    float pa = 0.0f, pb = 0.0f;
    if (i < d.nx && j < d.ny) {
        const int im = nb_lo(i, d.nx), ip = nb_hi(i, d.nx), jm = nb_lo(j, d.ny), jp = nb_hi(j, d.ny);
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            const float w = ldg(W, v);
            const float lx = ldg(W, vid(d, im, j, k)) + ldg(W, vid(d, ip, j, k)) - 2.0f * w;
            const float ly = ldg(W, vid(d, i, jm, k)) + ldg(W, vid(d, i, jp, k)) - 2.0f * w;
            float lap = lx + ly;
            if (THREE) {
                const float lz = ldg(W, vid(d, i, j, nb_lo(k, d.nz))) + ldg(W, vid(d, i, j, nb_hi(k, d.nz))) - 2.0f * w;
                lap = lap + lz;
            }
            const float u = U[v];
            const float un = u + tau * (-lam * lap - (u - ldg(F, v)));
            U[v] = un;
            if (check) {
                const float df = un - u;
                pa += df * df;
                pb += un * un;
            }
        }
    }
    if (check) block_pair_partial<256>(pa, pb, partials, block_slot());
}

}  // namespace

int diff4th_run(const float* f, float* u_out, float lam, float sigma, int iters, float tau, float epsil,
                const Dims& d, cudaStream_t s, float* info) {
    CILREG_RANGE("cilreg Diff4th");
    const bool three = d.nz > 1;
    Scratch scratch(s);
    const Launch3 L = plan_launch(d);
    // CILREG_D4_KERNEL=simple selects the two per-voxel kernels (kept for A/B checks)
    const char* ek = getenv("CILREG_D4_KERNEL");
    const bool stream = !(ek && strcmp(ek, "simple") == 0);
    const D4Plan T = d4_stream_plan(d);
    IterControl ctl(s, scratch, iters, epsil, stream ? T.nblocks : num_blocks(L));
    CILREG_TRY(ctl.status());
    float* W = scratch.floats(d.n);
    if (!W) return scratch.status();
    CILREG_CUDA(cudaMemcpyAsync(u_out, f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    const float sg2 = sigma * sigma;  // Diffus4th_order_core.c:51
    const float isg2 = 1.0f / sg2;    // den / sg2 formed as den * isg2 (within 1 ulp)
    if (stream) {
        // fused iteration, ping-pong between u_out and W's buffer
        float* bufs[2] = {u_out, W};
        int it = 0;
        if (!ctl.checking() && d.n <= (1LL << 22)) {
            // small volume, fixed count: launch overhead dominates, replay a graph
            CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
                CILREG_TRY(d4_stream_step(T, bufs[k & 1], bufs[(k + 1) & 1], f, lam, tau, isg2, d, ctl.ctl(), 0,
                                          ctl.partials(), st));
                note_launch();
                return OK;
            }));
            it = iters;
        }
        for (; it < iters; it++) {
            const int check = ctl.is_check(it) ? 1 : 0;
            CILREG_TRY(d4_stream_step(T, bufs[it & 1], bufs[(it + 1) & 1], f, lam, tau, isg2, d, ctl.ctl(), check,
                                      ctl.partials(), s));
            note_launch();
            if (check) {
                CILREG_TRY(ctl.after_check(it, T.nblocks));
                if (ctl.host_should_stop()) break;
            }
        }
        if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl.ctl(), iters, bufs, u_out, d.n, s));
        return ctl.finish(info);
    }
    int it = 0;
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        if (three) {
            k_d4_laplacian<true><<<L.grid, L.block, 0, s>>>(u_out, W, isg2, d, L.kz, ctl.ctl());
            k_d4_update<true><<<L.grid, L.block, 0, s>>>(u_out, W, f, lam, tau, d, L.kz, ctl.ctl(), check,
                                                         ctl.partials());
        } else {
            k_d4_laplacian<false><<<L.grid, L.block, 0, s>>>(u_out, W, isg2, d, L.kz, ctl.ctl());
            k_d4_update<false><<<L.grid, L.block, 0, s>>>(u_out, W, f, lam, tau, d, L.kz, ctl.ctl(), check,
                                                          ctl.partials());
        }
        CILREG_CUDA(cudaGetLastError());
        note_launch(2);
        if (check) {
            CILREG_TRY(ctl.after_check(it, num_blocks(L)));
            if (ctl.host_should_stop()) break;
        }
    }
    return ctl.finish(info);
}

}  // namespace cilreg
