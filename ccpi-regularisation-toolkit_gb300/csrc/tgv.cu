// TGV^2-L2 primal-dual denoising (reference: TGV_core.c:43-568).
//
// Two kernels per iteration, both in place (each voxel writes only itself):
//   k_tgv_dual    P += sigma (grad U - V), |P| <= alpha1;
//                 Q += sigma sym-grad V,   |Q|_F <= alpha0   (reads U, V at +1)
//   k_tgv_primal  U <- 2 prox(U + tau div P) - U;  V <- 2 (V + tau (P + div Q)) - V
//                 (reads P, Q at -1)
// Volumes below 2^31 voxels run 2.5D streaming versions of both (tgv_tiled.cu)
// unless CILREG_TGV_KERNEL=simple.
// 3D state: U, P(3), Q(6), V(3) plus U0.  The dual and primal halves of the
// reference's ten sweeps (TGV_core.c:136-167) collapse into these two.
#include <vector>

#include "drivers.cuh"
#include "tgv_batch.cuh"
#include "tgv_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {

namespace {


template <bool THREE>
__device__ __forceinline__ void tgv_dual_tile(const TgvArgs& a, const Dims& d, int kz, int bx, int by, int bz) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k0 = bz * kz;
    if (i >= d.nx || j >= d.ny) return;
    const bool xe = (i == d.nx - 1), ye = (j == d.ny - 1);
    for (int kk = 0; kk < kz; kk++) {
        const int k = k0 + kk;
        if (k >= d.nz) break;
        const bool ze = (k == d.nz - 1);
        const long long v = vid(d, i, j, k);
        const long long vx = v + 1, vy = v + d.nx, vz = v + d.sxy;
        const float u = a.u[v];
        const float v1 = a.v[0][v], v2 = a.v[1][v], v3 = THREE ? a.v[2][v] : 0.0f;
        // DualP (TGV_core.c:351-368)
        float p1 = a.p[0][v] + (xe ? a.sigma * (-v1) : a.sigma * ((a.u[vx] - u) - v1));
        float p2 = a.p[1][v] + (ye ? a.sigma * (-v2) : a.sigma * ((a.u[vy] - u) - v2));
        float p3 = 0.0f;
        if (THREE) p3 = a.p[2][v] + (ze ? a.sigma * (-v3) : a.sigma * ((a.u[vz] - u) - v3));
        // ProjP (TGV_core.c:370-387)
        const float gp = (THREE ? sqrtf(p1 * p1 + p2 * p2 + p3 * p3) : sqrtf(p1 * p1 + p2 * p2)) / a.alpha1;
        if (gp > 1.0f) {
            const float ig = __frcp_rn(gp);  // one reciprocal instead of three divisions
            p1 *= ig;
            p2 *= ig;
            p3 *= ig;
        }
        a.p[0][v] = p1;
        a.p[1][v] = p2;
        if (THREE) a.p[2][v] = p3;
        // DualQ + ProjQ (TGV_core.c:389-446 / 234-275)
        if (THREE) {
            float q1 = 0, q11 = 0, q33 = 0, q2 = 0, q22 = 0, q55 = 0, q3 = 0, q44 = 0, q66 = 0;
            if (!xe) { q1 = a.v[0][vx] - v1; q11 = a.v[1][vx] - v2; q33 = a.v[2][vx] - v3; }
            if (!ye) { q2 = a.v[1][vy] - v2; q22 = a.v[0][vy] - v1; q55 = a.v[2][vy] - v3; }
            if (!ze) { q3 = a.v[2][vz] - v3; q44 = a.v[0][vz] - v1; q66 = a.v[1][vz] - v2; }
            float Q1 = a.q[0][v] + a.sigma * q1;
            float Q2 = a.q[1][v] + a.sigma * q2;
            float Q3 = a.q[2][v] + a.sigma * q3;
            float Q4 = a.q[3][v] + a.sigma * (0.5f * (q11 + q22));
            float Q5 = a.q[4][v] + a.sigma * (0.5f * (q33 + q44));
            float Q6 = a.q[5][v] + a.sigma * (0.5f * (q55 + q66));
            float g = sqrtf(Q1 * Q1 + Q2 * Q2 + Q3 * Q3 + 2.0f * Q4 * Q4 + 2.0f * Q5 * Q5 + 2.0f * Q6 * Q6);
            g = g / a.alpha0;
            if (g > 1.0f) {
                const float ig = __frcp_rn(g);
                Q1 *= ig; Q2 *= ig; Q3 *= ig; Q4 *= ig; Q5 *= ig; Q6 *= ig;
            }
            a.q[0][v] = Q1; a.q[1][v] = Q2; a.q[2][v] = Q3;
            a.q[3][v] = Q4; a.q[4][v] = Q5; a.q[5][v] = Q6;
        } else {
            float q1 = 0, q11 = 0, q2 = 0, q22 = 0;
            if (!xe) { q1 = a.v[0][vx] - v1; q11 = a.v[1][vx] - v2; }
            if (!ye) { q2 = a.v[1][vy] - v2; q22 = a.v[0][vy] - v1; }
            float Q1 = a.q[0][v] + a.sigma * q1;
            float Q2 = a.q[1][v] + a.sigma * q2;
            float Q3 = a.q[2][v] + a.sigma * (0.5f * (q11 + q22));
            float g = sqrtf(Q1 * Q1 + Q2 * Q2 + 2.0f * Q3 * Q3);
            g = g / a.alpha0;
            if (g > 1.0f) {
                const float ig = __frcp_rn(g);
                Q1 *= ig; Q2 *= ig; Q3 *= ig;
            }
            a.q[0][v] = Q1; a.q[1][v] = Q2; a.q[2][v] = Q3;
        }
    }
}


// backward difference with the reference's three-case boundary (TGV_core.c:286-292)
__device__ __forceinline__ float bwd(const float* X, long long v, long long stride, int i, int n) {
    if (i == 0) return X[v];
    if (i == n - 1) return -X[v - stride];
    return X[v] - X[v - stride];
}

template <bool THREE>
__device__ __forceinline__ void tgv_primal_tile(const TgvArgs& a, const Dims& d, int kz, int bx, int by, int bz,
                                                float& pa, float& pb) {
    const int i = bx * 32 + threadIdx.x;
    const int j = by * 8 + threadIdx.y;
    const int k0 = bz * kz;
    if (i < d.nx && j < d.ny) {
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            // DivProjP + newU (TGV_core.c:448-472, 548-554)
            float dv = bwd(a.p[0], v, 1, i, d.nx) + bwd(a.p[1], v, d.nx, j, d.ny);
            if (THREE) dv = dv + bwd(a.p[2], v, d.sxy, k, d.nz);
            const float uo = a.u[v];
            const float un = (a.lambda * (uo + a.tau * dv) + a.tau * ldg(a.u0, v)) * a.inv_lt;
            const float ue = 2.0f * un - uo;
            a.u[v] = ue;
            if (a.check) {
                const float df = ue - uo;
                pa += df * df;
                pb += ue * ue;
            }
            // UpdV + newV (TGV_core.c:474-533, 558-568)
            if (THREE) {
                const float q1 = bwd(a.q[0], v, 1, i, d.nx), q4x = bwd(a.q[3], v, 1, i, d.nx),
                            q5x = bwd(a.q[4], v, 1, i, d.nx);
                const float q2 = bwd(a.q[1], v, d.nx, j, d.ny), q4y = bwd(a.q[3], v, d.nx, j, d.ny),
                            q6y = bwd(a.q[5], v, d.nx, j, d.ny);
                const float q6z = bwd(a.q[5], v, d.sxy, k, d.nz), q5z = bwd(a.q[4], v, d.sxy, k, d.nz),
                            q3 = bwd(a.q[2], v, d.sxy, k, d.nz);
                const float d1 = q1 + q4y + q5z, d2 = q4x + q2 + q6z, d3 = q5x + q6y + q3;
                const float v1 = a.v[0][v], v2 = a.v[1][v], v3 = a.v[2][v];
                a.v[0][v] = 2.0f * (v1 + a.tau * (a.p[0][v] + d1)) - v1;
                a.v[1][v] = 2.0f * (v2 + a.tau * (a.p[1][v] + d2)) - v2;
                a.v[2][v] = 2.0f * (v3 + a.tau * (a.p[2][v] + d3)) - v3;
            } else {
                const float q1 = bwd(a.q[0], v, 1, i, d.nx), q3x = bwd(a.q[2], v, 1, i, d.nx);
                const float q2 = bwd(a.q[1], v, d.nx, j, d.ny), q3y = bwd(a.q[2], v, d.nx, j, d.ny);
                const float d1 = q1 + q3y, d2 = q3x + q2;
                const float v1 = a.v[0][v], v2 = a.v[1][v];
                a.v[0][v] = 2.0f * (v1 + a.tau * (a.p[0][v] + d1)) - v1;
                a.v[1][v] = 2.0f * (v2 + a.tau * (a.p[1][v] + d2)) - v2;
            }
        }
    }
}


// single-volume kernels: the kernel parameter struct is read directly (a
// reference to it would copy the whole struct into registers)
template <bool THREE>
__global__ void __launch_bounds__(256) k_tgv_dual(TgvArgs a, Dims d, int kz, const StopCtl* ctl) {
    if (ctl->stop) return;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    if (i >= d.nx || j >= d.ny) return;
    const bool xe = (i == d.nx - 1), ye = (j == d.ny - 1);
    for (int kk = 0; kk < kz; kk++) {
        const int k = k0 + kk;
        if (k >= d.nz) break;
        const bool ze = (k == d.nz - 1);
        const long long v = vid(d, i, j, k);
        const long long vx = v + 1, vy = v + d.nx, vz = v + d.sxy;
        const float u = a.u[v];
        const float v1 = a.v[0][v], v2 = a.v[1][v], v3 = THREE ? a.v[2][v] : 0.0f;
        // DualP (TGV_core.c:351-368)
        float p1 = a.p[0][v] + (xe ? a.sigma * (-v1) : a.sigma * ((a.u[vx] - u) - v1));
        float p2 = a.p[1][v] + (ye ? a.sigma * (-v2) : a.sigma * ((a.u[vy] - u) - v2));
        float p3 = 0.0f;
        if (THREE) p3 = a.p[2][v] + (ze ? a.sigma * (-v3) : a.sigma * ((a.u[vz] - u) - v3));
        // ProjP (TGV_core.c:370-387)
        const float gp = (THREE ? sqrtf(p1 * p1 + p2 * p2 + p3 * p3) : sqrtf(p1 * p1 + p2 * p2)) / a.alpha1;
        if (gp > 1.0f) {
            const float ig = __frcp_rn(gp);  // one reciprocal instead of three divisions
            p1 *= ig;
            p2 *= ig;
            p3 *= ig;
        }
        a.p[0][v] = p1;
        a.p[1][v] = p2;
        if (THREE) a.p[2][v] = p3;
        // DualQ + ProjQ (TGV_core.c:389-446 / 234-275)
        if (THREE) {
            float q1 = 0, q11 = 0, q33 = 0, q2 = 0, q22 = 0, q55 = 0, q3 = 0, q44 = 0, q66 = 0;
            if (!xe) { q1 = a.v[0][vx] - v1; q11 = a.v[1][vx] - v2; q33 = a.v[2][vx] - v3; }
            if (!ye) { q2 = a.v[1][vy] - v2; q22 = a.v[0][vy] - v1; q55 = a.v[2][vy] - v3; }
            if (!ze) { q3 = a.v[2][vz] - v3; q44 = a.v[0][vz] - v1; q66 = a.v[1][vz] - v2; }
            float Q1 = a.q[0][v] + a.sigma * q1;
            float Q2 = a.q[1][v] + a.sigma * q2;
            float Q3 = a.q[2][v] + a.sigma * q3;
            float Q4 = a.q[3][v] + a.sigma * (0.5f * (q11 + q22));
            float Q5 = a.q[4][v] + a.sigma * (0.5f * (q33 + q44));
            float Q6 = a.q[5][v] + a.sigma * (0.5f * (q55 + q66));
            float g = sqrtf(Q1 * Q1 + Q2 * Q2 + Q3 * Q3 + 2.0f * Q4 * Q4 + 2.0f * Q5 * Q5 + 2.0f * Q6 * Q6);
            g = g / a.alpha0;
            if (g > 1.0f) {
                const float ig = __frcp_rn(g);
                Q1 *= ig; Q2 *= ig; Q3 *= ig; Q4 *= ig; Q5 *= ig; Q6 *= ig;
            }
            a.q[0][v] = Q1; a.q[1][v] = Q2; a.q[2][v] = Q3;
            a.q[3][v] = Q4; a.q[4][v] = Q5; a.q[5][v] = Q6;
        } else {
            float q1 = 0, q11 = 0, q2 = 0, q22 = 0;
            if (!xe) { q1 = a.v[0][vx] - v1; q11 = a.v[1][vx] - v2; }
            if (!ye) { q2 = a.v[1][vy] - v2; q22 = a.v[0][vy] - v1; }
            float Q1 = a.q[0][v] + a.sigma * q1;
            float Q2 = a.q[1][v] + a.sigma * q2;
            float Q3 = a.q[2][v] + a.sigma * (0.5f * (q11 + q22));
            float g = sqrtf(Q1 * Q1 + Q2 * Q2 + 2.0f * Q3 * Q3);
            g = g / a.alpha0;
            if (g > 1.0f) {
                const float ig = __frcp_rn(g);
                Q1 *= ig; Q2 *= ig; Q3 *= ig;
            }
            a.q[0][v] = Q1; a.q[1][v] = Q2; a.q[2][v] = Q3;
        }
    }
}

template <bool THREE>
__global__ void __launch_bounds__(256, 6) k_tgv_primal(TgvArgs a, Dims d, int kz, const StopCtl* ctl,
                                                    double2* partials) {
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
            // DivProjP + newU (TGV_core.c:448-472, 548-554)
            float dv = bwd(a.p[0], v, 1, i, d.nx) + bwd(a.p[1], v, d.nx, j, d.ny);
            if (THREE) dv = dv + bwd(a.p[2], v, d.sxy, k, d.nz);
            const float uo = a.u[v];
            const float un = (a.lambda * (uo + a.tau * dv) + a.tau * ldg(a.u0, v)) * a.inv_lt;
            const float ue = 2.0f * un - uo;
            a.u[v] = ue;
            if (a.check) {
                const float df = ue - uo;
                pa += df * df;
                pb += ue * ue;
            }
            // UpdV + newV (TGV_core.c:474-533, 558-568)
            if (THREE) {
                const float q1 = bwd(a.q[0], v, 1, i, d.nx), q4x = bwd(a.q[3], v, 1, i, d.nx),
                            q5x = bwd(a.q[4], v, 1, i, d.nx);
                const float q2 = bwd(a.q[1], v, d.nx, j, d.ny), q4y = bwd(a.q[3], v, d.nx, j, d.ny),
                            q6y = bwd(a.q[5], v, d.nx, j, d.ny);
                const float q6z = bwd(a.q[5], v, d.sxy, k, d.nz), q5z = bwd(a.q[4], v, d.sxy, k, d.nz),
                            q3 = bwd(a.q[2], v, d.sxy, k, d.nz);
                const float d1 = q1 + q4y + q5z, d2 = q4x + q2 + q6z, d3 = q5x + q6y + q3;
                const float v1 = a.v[0][v], v2 = a.v[1][v], v3 = a.v[2][v];
                a.v[0][v] = 2.0f * (v1 + a.tau * (a.p[0][v] + d1)) - v1;
                a.v[1][v] = 2.0f * (v2 + a.tau * (a.p[1][v] + d2)) - v2;
                a.v[2][v] = 2.0f * (v3 + a.tau * (a.p[2][v] + d3)) - v3;
            } else {
                const float q1 = bwd(a.q[0], v, 1, i, d.nx), q3x = bwd(a.q[2], v, 1, i, d.nx);
                const float q2 = bwd(a.q[1], v, d.nx, j, d.ny), q3y = bwd(a.q[2], v, d.nx, j, d.ny);
                const float d1 = q1 + q3y, d2 = q3x + q2;
                const float v1 = a.v[0][v], v2 = a.v[1][v];
                a.v[0][v] = 2.0f * (v1 + a.tau * (a.p[0][v] + d1)) - v1;
                a.v[1][v] = 2.0f * (v2 + a.tau * (a.p[1][v] + d2)) - v2;
            }
        }
    }
    if (a.check) block_pair_partial<256>(pa, pb, partials, block_slot());
}

// batched: one flat grid over the tiles of every volume
template <bool THREE>
__global__ void __launch_bounds__(256, 4) k_tgv_dual_batch(const TgvBatchVol* __restrict__ vols,
                                                        const int* __restrict__ tile_vol) {
    const long long t = blockIdx.x;
    const TgvBatchVol& V = vols[tile_vol[t]];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    TgvArgs a = V.args;
    tgv_dual_tile<THREE>(a, V.d, V.kz, (int)(lt % V.gx), (int)((lt / V.gx) % V.gy),
                         (int)(lt / ((long long)V.gx * V.gy)));
}

template <bool THREE>
__global__ void __launch_bounds__(256, 4) k_tgv_primal_batch(const TgvBatchVol* __restrict__ vols,
                                                          const int* __restrict__ tile_vol, int check) {
    const long long t = blockIdx.x;
    const TgvBatchVol& V = vols[tile_vol[t]];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    TgvArgs a = V.args;
    a.check = check;
    float pa = 0.0f, pb = 0.0f;
    tgv_primal_tile<THREE>(a, V.d, V.kz, (int)(lt % V.gx), (int)((lt / V.gx) % V.gy),
                           (int)(lt / ((long long)V.gx * V.gy)), pa, pb);
    if (check) block_pair_partial<256>(pa, pb, V.partials, lt);
}

}  // namespace

int tgv_batch_step(const TgvBatchVol* d_vols, const int* d_tile_vol, long long ntiles, const int* d_ptile_vol,
                   long long nptiles, bool three, int check, cudaStream_t s) {
    if (ntiles < 1 || ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", ntiles);
    if (d_ptile_vol) {
        CILREG_TRY(tgv_dual_batch_step(d_vols, d_ptile_vol, nptiles, three, s));
        return tgv_primal_batch_step(d_vols, d_ptile_vol, nptiles, three, check, s);
    }
    const dim3 grid((unsigned)ntiles), block(32, 8, 1);
    if (three) k_tgv_dual_batch<true><<<grid, block, 0, s>>>(d_vols, d_tile_vol);
    else k_tgv_dual_batch<false><<<grid, block, 0, s>>>(d_vols, d_tile_vol);
    CILREG_CUDA(cudaGetLastError());
    if (three) k_tgv_primal_batch<true><<<grid, block, 0, s>>>(d_vols, d_tile_vol, check);
    else k_tgv_primal_batch<false><<<grid, block, 0, s>>>(d_vols, d_tile_vol, check);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

namespace {

// 3D: one fused pass per iteration over double-buffered U, V, P, Q
int tgv_run_fused(const float* f, float* u_out, float lam, float alpha1, float alpha0, int iters, float L2,
                  float epsil, const Dims& d, cudaStream_t s, float* info, const TgvPlan& T, Scratch& scratch) {
    IterControl ctl(s, scratch, iters, epsil, T.nblocks);
    CILREG_TRY(ctl.status());
    const size_t nb = sizeof(float) * (size_t)d.n;
    float* ub[2] = {u_out, scratch.floats(d.n)};
    float* vb[2][3] = {};
    float* pb[2][3] = {};
    float* qb[2][6] = {};
    if (!ub[1]) return scratch.status();
    for (int b = 0; b < 2; b++) {
        for (int c = 0; c < 3; c++) {
            vb[b][c] = scratch.floats(d.n);
            pb[b][c] = scratch.floats(d.n);
            if (!vb[b][c] || !pb[b][c]) return scratch.status();
        }
        for (int c = 0; c < 6; c++)
            if (!(qb[b][c] = scratch.floats(d.n))) return scratch.status();
    }
    // the initial state: U = U0, V = P = Q = 0 (calloc, TGV_core.c:57-70, 128-133)
    for (int c = 0; c < 3; c++) {
        CILREG_CUDA(cudaMemsetAsync(vb[0][c], 0, nb, s));
        CILREG_CUDA(cudaMemsetAsync(pb[0][c], 0, nb, s));
    }
    for (int c = 0; c < 6; c++) CILREG_CUDA(cudaMemsetAsync(qb[0][c], 0, nb, s));
    CILREG_CUDA(cudaMemcpyAsync(u_out, f, nb, cudaMemcpyDeviceToDevice, s));
    TgvFusedArgs a;
    a.u0 = f;
    a.lambda = lam;
    a.alpha1 = alpha1;
    a.alpha0 = alpha0;
    a.tau = (float)pow((double)L2, -0.5);  // TGV_core.c:54-55
    a.sigma = a.tau;
    a.inv_lt = 1.0f / (a.lambda + a.tau);
    // tensor maps of the staged pass, one set per buffer parity (the pass that
    // loads by threads runs on the same tiling if an array is misaligned)
    const size_t mb = tgv_tma_maps_bytes();
    std::vector<unsigned char> maps(T.tma ? 2 * mb : 0);
    bool tma = T.tma;
    auto set_parity = [&](int k) {
        const int cur = k & 1, nxt = cur ^ 1;
        a.u = ub[cur];
        a.un = ub[nxt];
        for (int c = 0; c < 3; c++) {
            a.v[c] = vb[cur][c];
            a.vn[c] = vb[nxt][c];
            a.p[c] = pb[cur][c];
            a.pn[c] = pb[nxt][c];
        }
        for (int c = 0; c < 6; c++) {
            a.q[c] = qb[cur][c];
            a.qn[c] = qb[nxt][c];
        }
    };
    for (int k = 0; k < 2 && tma; k++) {
        set_parity(k);
        tma = tgv_tma_encode(a, d, maps.data() + mb * k);
    }
    auto step = [&](int k, int check, cudaStream_t st) -> int {
        if (tma) return tgv_tma_step(T, maps.data() + mb * (k & 1), a, d, ctl.ctl(), check, ctl.partials(), st);
        return tgv_fused_step(T, a, d, ctl.ctl(), check, ctl.partials(), st);
    };
    int it = 0;
    if (!ctl.checking() && d.n <= (1LL << 22)) {
        // small volume, fixed count: launch overhead dominates, replay a graph
        CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
            set_parity(k);
            CILREG_TRY(step(k, 0, st));
            note_launch();
            return OK;
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        set_parity(it);
        CILREG_TRY(step(it, check, s));
        note_launch();
        if (check) {
            CILREG_TRY(ctl.after_check(it, T.nblocks));
            if (ctl.host_should_stop()) break;
        }
    }
    if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl.ctl(), iters, ub, u_out, d.n, s));
    if (tma) CILREG_TRY(tgv_tma_status(s));
    return ctl.finish(info);
}

}  // namespace

int tgv_run(const float* f, float* u_out, float lam, float alpha1, float alpha0, int iters, float L2, float epsil,
            const Dims& d, cudaStream_t s, float* info) {
    CILREG_RANGE("cilreg TGV");
    const bool three = d.nz > 1;
    const int np = three ? 3 : 2, nq = three ? 6 : 3;
    Scratch scratch(s);
    const Launch3 L = plan_launch(d);
    const TgvPlan T = tgv_primal_plan(d);
    const TgvPlan TF = T.use ? tgv_fused_plan(d) : TgvPlan{};
    if (TF.use) return tgv_run_fused(f, u_out, lam, alpha1, alpha0, iters, L2, epsil, d, s, info, TF, scratch);
    const long long nparts = T.use ? T.nblocks : num_blocks(L);
    IterControl ctl(s, scratch, iters, epsil, nparts);
    CILREG_TRY(ctl.status());
    TgvArgs a;
    for (int c = 0; c < 3; c++) { a.p[c] = nullptr; a.v[c] = nullptr; }
    for (int c = 0; c < 6; c++) a.q[c] = nullptr;
    for (int c = 0; c < np; c++) {
        a.p[c] = scratch.floats(d.n);
        a.v[c] = scratch.floats(d.n);
        if (!a.p[c] || !a.v[c]) return scratch.status();
        CILREG_CUDA(cudaMemsetAsync(a.p[c], 0, sizeof(float) * d.n, s));
        CILREG_CUDA(cudaMemsetAsync(a.v[c], 0, sizeof(float) * d.n, s));
    }
    for (int c = 0; c < nq; c++) {
        a.q[c] = scratch.floats(d.n);
        if (!a.q[c]) return scratch.status();
        CILREG_CUDA(cudaMemsetAsync(a.q[c], 0, sizeof(float) * d.n, s));
    }
    CILREG_CUDA(cudaMemcpyAsync(u_out, f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    a.u = u_out;
    a.u0 = f;
    a.lambda = lam;
    a.alpha1 = alpha1;
    a.alpha0 = alpha0;
    a.tau = (float)pow((double)L2, -0.5);  // TGV_core.c:54-55
    a.sigma = a.tau;
    a.inv_lt = 1.0f / (a.lambda + a.tau);
    int it = 0;
    if (T.use && !ctl.checking() && d.n <= (1LL << 22)) {
        // small volume (2D here), fixed count: launch overhead dominates, replay a graph
        a.check = 0;
        CILREG_TRY(run_replayed(iters, 64, s, [&](int, cudaStream_t st, bool) -> int {
            CILREG_TRY(tgv_dual_stream_step(T, a, d, ctl.ctl(), st));
            CILREG_TRY(tgv_primal_stream_step(T, a, d, ctl.ctl(), ctl.partials(), st));
            note_launch(2);
            return OK;
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        a.check = check;
        if (T.use) {
            CILREG_TRY(tgv_dual_stream_step(T, a, d, ctl.ctl(), s));
            CILREG_TRY(tgv_primal_stream_step(T, a, d, ctl.ctl(), ctl.partials(), s));
        } else {
            if (three) k_tgv_dual<true><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl());
            else k_tgv_dual<false><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl());
            CILREG_CUDA(cudaGetLastError());
            if (three) k_tgv_primal<true><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
            else k_tgv_primal<false><<<L.grid, L.block, 0, s>>>(a, d, L.kz, ctl.ctl(), ctl.partials());
            CILREG_CUDA(cudaGetLastError());
        }
        note_launch(2);
        if (check) {
            CILREG_TRY(ctl.after_check(it, nparts));
            if (ctl.host_should_stop()) break;
        }
    }
    return ctl.finish(info);
}

}  // namespace cilreg
