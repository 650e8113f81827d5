// One whole TGV iteration (dual and primal halves, TGV_core.c:351-568) in one
// 2.5D streaming pass for 3D volumes.
//
// The dual half needs U and V at the forward neighbours, the primal half the
// new P and Q at the backward neighbours, so a tile has a one-voxel halo on
// both sides: thread (tx, ty) sits on voxel (x0 - 1 + tx, y0 - 1 + ty), the
// dual is formed for tx <= 30, ty <= 14 and the primal on the inner 30 x 14.
// The state is double-buffered (a neighbouring tile's halo still reads the
// old U, V, P, Q): the pass reads U, V (3), P (3), Q (6) and U0 and writes the
// new U, V, P, Q, 108 B per voxel against 88 + 72 B for the two streaming
// half-iteration passes (tgv_tiled.cu).  Step j of each thread, walking a z
// chunk (j from its first plane - 1):
//   1. publishes U, V of plane j (loaded two steps ahead, the z successor is
//      in registers);
//   2. (barrier) forms the new P, Q of plane j with the forward differences
//      and projections of the dual half, writes them, and publishes the
//      components the x/y successors' divergences need;
//   3. (barrier) forms the new U, V of plane j from the backward divergences
//      of the new P, Q (z predecessor in registers), extrapolates and writes
//      them.
// Every expression is the one of tgv_tiled.cu, so the pass gives the two
// passes' iterates bit for bit.
#include <type_traits>

#include "tgv_fused_math.cuh"
#include "tgv_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 2, OY = BY - 2;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

// One tile (bx, by, bz) of one volume; A is the argument block, a kernel
// parameter or (batched runs) a volatile copy in shared memory, read at each
// use rather than held in registers.
template <bool CHECK, class A>
__device__ __forceinline__ void fused_tile(A& a, const Dims& d, int zc, int bx, int by, int bz, float& pa_out,
                                           float& pb_out) {
    __shared__ float sUV[4][BY * BX];  // U, V1..V3 of plane j
    __shared__ float sPQ[7][BY * BX];  // new P1, P2, Q1, Q2, Q4, Q5, Q6 of plane j
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = bx * OX + tx - 1;
    const int y = by * OY + ty - 1;
    const int z0 = bz * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool d_pt = in_xy && tx <= BX - 2 && ty <= BY - 2;   // dual formed here
    const bool o_pt = d_pt && tx >= 1 && ty >= 1;                // primal formed and written here
    const bool xe = (x == nx - 1), ye = (y == ny - 1), xf = (x == 0), yf = (y == 0);
    const int oc = ty * BX + tx;
    const int oxh = ty * BX + min(tx + 1, BX - 1), oyh = min(ty + 1, BY - 1) * BX + tx;
    const int oxl = ty * BX + max(tx - 1, 0), oyl = max(ty - 1, 0) * BX + tx;
    const int col = min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const int sxy = (int)d.sxy;
    auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
    const float sigma = a.sigma, tau = a.tau, lam = a.lambda, ilt = a.inv_lt;
    const float alpha1 = a.alpha1, alpha0 = a.alpha0;
    auto ld_uv = [&](int k, float* w) {
        const int o = at(k);
        w[0] = __ldg(a.u + o);
        for (int i = 0; i < 3; i++) w[1 + i] = __ldg(a.v[i] + o);
    };
    float cw[4], nw[4];  // U, V1..V3 of planes j and j+1
    ld_uv(z0 - 1, cw);
    ld_uv(z0, nw);
    // new P3, Q3, Q5, Q6 of plane j-1 (z predecessors of the divergences)
    float zp3 = 0.f, zq3 = 0.f, zq5 = 0.f, zq6 = 0.f;
    float pa = 0.f, pb = 0.f;

    for (int j = z0 - 1; j < z1; ++j) {
        float fw[4];  // plane j+2, used two steps on
        ld_uv(j + 2, fw);
        const bool plane_ok = (j >= 0);
        const int o = (plane_ok ? j : 0) * sxy + col;
        float pq[9];
        if (d_pt && plane_ok)
            for (int i = 0; i < 3; i++) pq[i] = __ldg(a.p[i] + o);
        if (d_pt && plane_ok)
            for (int i = 0; i < 6; i++) pq[3 + i] = __ldg(a.q[i] + o);
        const float u0 = (o_pt && j >= z0) ? __ldg(a.u0 + o) : 0.f;
        // 1. publish U, V of plane j
        for (int i = 0; i < 4; i++) sUV[i][oc] = cw[i];
        __syncthreads();
        // 2. dual half at plane j (DualP_3D + ProjP_3D, DualQ_3D + ProjQ_3D)
        TgvDual n{};
        if (d_pt && plane_ok) {
            n = tgv_dual_voxel(
                cw[0], cw[1], cw[2], cw[3], [&](int c) { return sUV[c][oxh]; }, [&](int c) { return sUV[c][oyh]; },
                [&](int c) { return nw[c]; }, pq, xe, ye, j == nz - 1, sigma, alpha1, alpha0);
            if (o_pt && j >= z0) {
                a.pn[0][o] = n.p1;
                a.pn[1][o] = n.p2;
                a.pn[2][o] = n.p3;
                a.qn[0][o] = n.q1;
                a.qn[1][o] = n.q2;
                a.qn[2][o] = n.q3;
                a.qn[3][o] = n.q4;
                a.qn[4][o] = n.q5;
                a.qn[5][o] = n.q6;
            }
        }
        sPQ[0][oc] = n.p1;
        sPQ[1][oc] = n.p2;
        sPQ[2][oc] = n.q1;
        sPQ[3][oc] = n.q2;
        sPQ[4][oc] = n.q4;
        sPQ[5][oc] = n.q5;
        sPQ[6][oc] = n.q6;
        __syncthreads();
        // 3. primal half at plane j (DivProjP_3D + newU3D, UpdV_3D + newV)
        if (o_pt && j >= z0) {
            const bool zf = (j == 0), zl = (j == nz - 1);
            const float ue = tgv_primal_u(n, sPQ[0][oxl], sPQ[1][oyl], zp3, xf, xe, yf, ye, zf, zl, cw[0], u0, lam,
                                          tau, ilt);
            a.un[o] = ue;
            if (CHECK) {
                const float df = ue - cw[0];
                pa += df * df;
                pb += ue * ue;
            }
            const TgvNewV w = tgv_primal_v(n, sPQ[2][oxl], sPQ[4][oxl], sPQ[5][oxl], sPQ[3][oyl], sPQ[4][oyl],
                                           sPQ[6][oyl], zq3, zq5, zq6, xf, xe, yf, ye, zf, zl, cw[1], cw[2], cw[3], tau);
            a.vn[0][o] = w.v1;
            a.vn[1][o] = w.v2;
            a.vn[2][o] = w.v3;
        }
        zp3 = n.p3;
        zq3 = n.q3;
        zq5 = n.q5;
        zq6 = n.q6;
        for (int i = 0; i < 4; i++) {
            cw[i] = nw[i];
            nw[i] = fw[i];
        }
    }
    pa_out = pa;
    pb_out = pb;
}

template <bool CHECK>
__global__ void __launch_bounds__(NT, 2) k_tgv_fused(TgvFusedArgs a, Dims d, int zc, const StopCtl* ctl,
                                                     double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    float pa = 0.f, pb = 0.f;
    fused_tile<CHECK, const TgvFusedArgs>(a, d, zc, blockIdx.x, blockIdx.y, blockIdx.z, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// one iteration of every volume of a batch: a flat grid over all volumes'
// tiles; `parity` selects the (old, new) buffer pair of the iteration
template <bool CHECK>
__global__ void __launch_bounds__(NT, 2) k_tgv_fused_batch(const TgvFusedVol* __restrict__ vols,
                                                           const int* __restrict__ tile_vol, int parity) {
    __shared__ TgvFusedArgs sa;
    const long long t = blockIdx.x;
    const TgvFusedVol& V = vols[tile_vol[t]];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    const int bx = (int)(lt % V.gx);
    const int by = (int)((lt / V.gx) % V.gy);
    const int bz = (int)(lt / ((long long)V.gx * V.gy));
    if (threadIdx.x == 0 && threadIdx.y == 0) sa = V.args[parity];
    __syncthreads();
    const volatile TgvFusedArgs& va = sa;
    float pa = 0.f, pb = 0.f;
    fused_tile<CHECK, const volatile TgvFusedArgs>(va, V.d, V.zc, bx, by, bz, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, V.partials, lt);
}

}  // namespace

TgvPlan tgv_fused_plan(const Dims& d) {
    TgvPlan T;
    const char* e = getenv("CILREG_TGV_FUSED");
    T.use = d.nz > 1 && d.n < (1LL << 31) && !(e && e[0] == '0');
    if (!T.use) return T;
    static const int resident = resident_ctas(k_tgv_fused<false>, NT);
    T.tma = tgv_tma_usable(d);
    T.block = dim3(BX, BY, 1);
    const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
    T.zchunk = wave_zchunk(tiles, d.nz, T.tma ? tgv_tma_resident() : resident, 1, ZCHUNK);
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

void tgv_fused_tiles(const Dims& d, int& gx, int& gy, int& gz, int& zc) {
    zc = (d.nz < ZCHUNK) ? d.nz : ZCHUNK;
    gx = (d.nx + OX - 1) / OX;
    gy = (d.ny + OY - 1) / OY;
    gz = (d.nz + zc - 1) / zc;
}

int tgv_fused_batch_step(const TgvFusedVol* d_vols, const int* d_tile_vol, long long ntiles, int parity, int check,
                         cudaStream_t s) {
    if (ntiles < 1 || ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", ntiles);
    if (check)
        k_tgv_fused_batch<true><<<dim3((unsigned)ntiles), dim3(BX, BY, 1), 0, s>>>(d_vols, d_tile_vol, parity);
    else
        k_tgv_fused_batch<false><<<dim3((unsigned)ntiles), dim3(BX, BY, 1), 0, s>>>(d_vols, d_tile_vol, parity);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int tgv_fused_step(const TgvPlan& T, const TgvFusedArgs& a, const Dims& d, const StopCtl* ctl, int check,
                   double2* partials, cudaStream_t s) {
    if (check)
        CILREG_CUDA(launch_pdl(k_tgv_fused<true>, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    else
        CILREG_CUDA(launch_pdl(k_tgv_fused<false>, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
