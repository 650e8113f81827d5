// ROF-TV explicit gradient flow (reference: ROF_TV_core.c:50-317).
//
// One fused kernel per iteration: the three normalised fluxes D1 (j axis),
// D2 (i axis), D3 (k axis) are evaluated on the fly at the voxel and at its
// mirrored lower neighbours, so neither D array is stored.  HBM traffic per
// voxel-iteration: read U and f, write U (12 B), ping-pong U buffers.
#include "drivers.cuh"
#include "rof_tiled.cuh"

#include <stdlib.h>
#include "nvtx.cuh"

namespace cilreg {

namespace {

__device__ __forceinline__ float minmod(float a, float b) {
    return 0.5f * (sgnf(a) + sgnf(b)) * fminf(fabsf(a), fabsf(b));
}

// flux along j ("x" in the reference naming), ROF_TV_core.c:122-137
template <bool THREE>
__device__ __forceinline__ float flux_j(const float* __restrict__ U, const Dims& d, int i, int j, int k) {
    const float a = ldg(U, vid(d, i, j, k));
    const float dp = ldg(U, vid(d, i, nb_hi(j, d.ny), k)) - a;
    const float xp = ldg(U, vid(d, nb_hi(i, d.nx), j, k)) - a;
    const float xm = a - ldg(U, vid(d, nb_lo(i, d.nx), j, k));
    float m = minmod(xp, xm);
    float s = dp * dp + m * m;
    if (THREE) {
        const float zp = ldg(U, vid(d, i, j, nb_hi(k, d.nz))) - a;
        const float zm = a - ldg(U, vid(d, i, j, nb_lo(k, d.nz)));
        m = minmod(zp, zm);
        s = s + m * m;
    }
    return dp / sqrtf(s + 1.0e-8f);
}

// flux along i ("y"), ROF_TV_core.c:187-200
template <bool THREE>
__device__ __forceinline__ float flux_i(const float* __restrict__ U, const Dims& d, int i, int j, int k) {
    const float a = ldg(U, vid(d, i, j, k));
    const float dp = ldg(U, vid(d, nb_hi(i, d.nx), j, k)) - a;
    const float yp = ldg(U, vid(d, i, nb_hi(j, d.ny), k)) - a;
    const float ym = a - ldg(U, vid(d, i, nb_lo(j, d.ny), k));
    float m = minmod(yp, ym);
    float s = dp * dp + m * m;
    if (THREE) {
        const float zp = ldg(U, vid(d, i, j, nb_hi(k, d.nz))) - a;
        const float zm = a - ldg(U, vid(d, i, j, nb_lo(k, d.nz)));
        m = minmod(zp, zm);
        s = s + m * m;
    }
    return dp / sqrtf(s + 1.0e-8f);
}

// flux along k ("z"), ROF_TV_core.c:250-263
__device__ __forceinline__ float flux_k(const float* __restrict__ U, const Dims& d, int i, int j, int k) {
    const float a = ldg(U, vid(d, i, j, k));
    const float dp = ldg(U, vid(d, i, j, nb_hi(k, d.nz))) - a;
    const float xp = ldg(U, vid(d, nb_hi(i, d.nx), j, k)) - a;
    const float xm = a - ldg(U, vid(d, nb_lo(i, d.nx), j, k));
    const float yp = ldg(U, vid(d, i, nb_hi(j, d.ny), k)) - a;
    const float ym = a - ldg(U, vid(d, i, nb_lo(j, d.ny), k));
    const float m1 = minmod(yp, ym), m2 = minmod(xp, xm);
    const float s = dp * dp + m1 * m1 + m2 * m2;
    return dp / sqrtf(s + 1.0e-8f);
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_rof_step(const float* __restrict__ U, float* __restrict__ Un,
                                                  const float* __restrict__ F, const float* __restrict__ lam_arr,
                                                  float lam, float tau, Dims d, int kz, const StopCtl* ctl,
                                                  int check, double2* partials) {
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
            const float u = ldg(U, v);
            const float l = lam_arr ? ldg(lam_arr, v) : lam;
            const float dv1 = flux_j<THREE>(U, d, i, j, k) - flux_j<THREE>(U, d, i, nb_lo(j, d.ny), k);
            const float dv2 = flux_i<THREE>(U, d, i, j, k) - flux_i<THREE>(U, d, nb_lo(i, d.nx), j, k);
            float div;
            if (THREE) {
                const float dv3 = flux_k(U, d, i, j, k) - flux_k(U, d, i, j, nb_lo(k, d.nz));
                div = dv1 + dv2 + dv3;
            } else {
                div = dv1 + dv2;
            }
            const float un = u + tau * (l * div - (u - ldg(F, v)));
            Un[v] = un;
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

namespace {
// CILREG_ROF_KERNEL=simple selects the per-voxel kernel (kept for A/B checks)
bool use_simple_kernel() {
    const char* e = getenv("CILREG_ROF_KERNEL");
    return e && e[0] == 's';
}
}  // namespace

long long rof_partial_slots(const Dims& d) {
    return use_simple_kernel() ? num_blocks(plan_launch(d)) : rof_tiled_plan(d).nblocks;
}

int rof_check_grid(const Dims& d) {
    const dim3 g = use_simple_kernel() ? plan_launch(d).grid : rof_tiled_plan(d).grid;
    if (g.y > 65535u || g.z > 65535u)
        return fail(ERR_ARG, __FILE__, __LINE__, "shape (%d, %d, %d) exceeds the launch grid (%u x %u x %u CTAs)",
                    d.nx, d.ny, d.nz, g.x, g.y, g.z);
    return OK;
}

int rof_launch_step(const float* cur, float* nxt, const float* f, const float* lam_arr, float lam, float tau,
                    const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    if (use_simple_kernel()) {
        const Launch3 L = plan_launch(d);
        if (d.nz > 1)
            k_rof_step<true><<<L.grid, L.block, 0, s>>>(cur, nxt, f, lam_arr, lam, tau, d, L.kz, ctl, check, partials);
        else
            k_rof_step<false><<<L.grid, L.block, 0, s>>>(cur, nxt, f, lam_arr, lam, tau, d, L.kz, ctl, check,
                                                         partials);
        CILREG_CUDA(cudaGetLastError());
    } else {
        CILREG_TRY(rof_tiled_step(rof_tiled_plan(d), cur, nxt, f, lam_arr, lam, tau, d, ctl, check, partials, s));
    }
    note_launch();
    return OK;
}

int rof_run(const float* f, float* u_out, const float* lam_arr, float lam, int iters, float tau, float epsil,
            const Dims& d, cudaStream_t s, float* info, const float* u_init) {
    CILREG_RANGE("cilreg ROF-TV");
    CILREG_TRY(rof_check_grid(d));
    Scratch scratch(s);
    const long long nparts = rof_partial_slots(d);
    IterControl ctl(s, scratch, iters, epsil, nparts);
    CILREG_TRY(ctl.status());
    float* alt = scratch.floats(d.n);
    if (!alt) return scratch.status();
    float* bufs[2] = {u_out, alt};
    CILREG_CUDA(cudaMemcpyAsync(u_out, u_init ? u_init : f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    int it = 0;
    if (!ctl.checking() && !use_simple_kernel() && rof_tb2d_depth(d, iters) == 0 &&
        rof_persist2d_applies(d, iters)) {
        // 2D image, fixed count: every iteration in one persistent launch
        const long long tiles = rof_persist2d_tiles(d);
        int* flags = (int*)scratch.bytes(sizeof(int) * (size_t)(tiles + 1));
        if (!flags) return scratch.status();
        CILREG_TRY(rof_persist2d_run(u_out, alt, f, lam_arr, lam, tau, iters, d, flags, flags + tiles, s));
        note_launch();
        int err = 0;
        CILREG_CUDA(cudaMemcpyAsync(&err, flags + tiles, sizeof(int), cudaMemcpyDeviceToHost, s));
        CILREG_CUDA(cudaStreamSynchronize(s));
        if (err) return fail(ERR_CUDA, __FILE__, __LINE__, "a wait between the tiles of k_rof_persist2d ran out");
        if (iters & 1) CILREG_CUDA(cudaMemcpyAsync(u_out, alt, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
        return ctl.finish(info);
    }
    const int depth = ctl.checking() ? 0 : rof_tb2d_depth(d, iters);
    if (depth > 0 && !use_simple_kernel()) {
        // 2D image, fixed count: `depth` iterations per launch on tiles with
        // overlapped halos; launches 0 .. nl-2 replayed from a graph, the
        // last one (the remaining iterations) directly
        const int nl = (iters + depth - 1) / depth;
        const int last = iters - (nl - 1) * depth;
        CILREG_TRY(run_replayed(nl - 1, 16, s, [&](int k, cudaStream_t st, bool) -> int {
            CILREG_TRY(rof_tb2d_step(bufs[k & 1], bufs[(k + 1) & 1], f, lam_arr, lam, tau, d, depth, st));
            note_launch();
            return OK;
        }));
        CILREG_TRY(rof_tb2d_step(bufs[(nl - 1) & 1], bufs[nl & 1], f, lam_arr, lam, tau, d, last, s));
        note_launch();
        if (nl & 1) CILREG_CUDA(cudaMemcpyAsync(u_out, alt, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
        return ctl.finish(info);
    }
    if (!ctl.checking() && d.n <= (1LL << 22)) {
        // small volume, fixed count: launch overhead dominates, replay a graph
        CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
            return rof_launch_step(bufs[k & 1], bufs[(k + 1) & 1], f, lam_arr, lam, tau, d, ctl.ctl(), 0, nullptr,
                                   st);
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        const float* cur = bufs[it & 1];
        float* nxt = bufs[(it + 1) & 1];
        CILREG_TRY(rof_launch_step(cur, nxt, f, lam_arr, lam, tau, d, ctl.ctl(), check, ctl.partials(), s));
        if (check) {
            CILREG_TRY(ctl.after_check(it, nparts));
            if (ctl.host_should_stop()) break;
        }
    }
    if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl.ctl(), iters, bufs, u_out, d.n, s));
    return ctl.finish(info);
}

}  // namespace cilreg
