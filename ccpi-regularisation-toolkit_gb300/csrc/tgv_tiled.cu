// TGV primal half-iteration (DivProjP + newU and UpdV + newV, reference
// TGV_core.c:277-345 in 2D, 448-568 in 3D) as a 2.5D streaming kernel.
//
// Every term is a backward difference of P or Q with the reference's
// three-case boundary rule (index 0: X; last index: -X[-1]; else X - X[-1]),
// so a tile needs a halo of one voxel on its low x and y sides only: thread
// (tx, ty) sits on voxel (x0 - 1 + tx, y0 - 1 + ty) and updates it when tx, ty
// >= 1 (31 x 15 voxels per 32 x 16 CTA).  Per plane each thread loads its
// voxel's P, Q, U, U0, V once (one plane ahead), publishes the P and Q
// components its x / y successors need to shared memory (two slots, one
// barrier per plane), keeps the z components of the previous plane in
// registers, and updates U and V in place (each voxel writes only itself and
// reads no other voxel's U or V).  HBM traffic: read P, Q, U, U0, V; write U,
// V (68 B per voxel in 3D, 44 B in 2D), against about 72 B for the per-voxel
// kernel and its cached neighbour loads.
#include <type_traits>

#include "tgv_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 1, OY = BY - 1;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

// backward difference with the three-case boundary (TGV_core.c:286-292)
__device__ __forceinline__ float bwd(float x, float xprev, bool first, bool last) {
    return first ? x : (last ? -xprev : x - xprev);
}

__device__ __forceinline__ void publish_args(const TgvArgs& a, float* volatile* tab, float* sc) {
    for (int i = 0; i < 3; i++) tab[i] = a.p[i];
    for (int i = 0; i < 6; i++) tab[3 + i] = a.q[i];
    for (int i = 0; i < 3; i++) tab[9 + i] = a.v[i];
    tab[12] = a.u;
    tab[13] = const_cast<float*>(a.u0);
    sc[0] = a.tau;
    sc[1] = a.lambda;
    sc[2] = a.inv_lt;
}

// BATCH: one flat grid over the tiles of every volume of a batched run
// (TgvBatchVol::pgx.. describe a volume's tiles); otherwise one volume.  The
// CTA copies its volume's arguments to shared memory first, so the state
// pointers are read from there rather than held in registers.
template <bool THREE, bool CHECK, bool BATCH>
__global__ void __launch_bounds__(NT, 2) k_tgv_primal_stream(TgvArgs a1, Dims d1, int zc1, const StopCtl* ctl1,
                                                             double2* partials1, const TgvBatchVol* __restrict__ vols,
                                                             const int* __restrict__ tile_vol) {
    // x/y predecessors: 3D P1 P2 Q1 Q2 Q4 Q5 Q6; 2D P1 P2 Q1 Q2 Q3
    constexpr int NS = THREE ? 7 : 5;
    __shared__ float sm[2][NS][BY * BX];
    // state pointers, read from shared memory at each use (volatile: not held
    // in registers across the loop); 0-2 P, 3-8 Q, 9-11 V, 12 U, 13 U0
    __shared__ float* volatile tab[14];
    __shared__ float sc[3];  // tau, lambda, 1 / (lambda + tau)
    int bx, by, bz, zc;
    Dims d;
    const StopCtl* ctl;
    double2* partials;
    long long slot;
    if constexpr (BATCH) {
        const long long t = blockIdx.x;
        const TgvBatchVol& V = vols[tile_vol[t]];
        const long long lt = t - V.ptile_base;
        bx = (int)(lt % V.pgx);
        by = (int)((lt / V.pgx) % V.pgy);
        bz = (int)(lt / ((long long)V.pgx * V.pgy));
        d = V.d;
        zc = V.pzc;
        ctl = V.ctl;
        partials = V.partials;
        slot = lt;
        if (threadIdx.x == 0 && threadIdx.y == 0) publish_args(V.args, tab, sc);
    } else {
        bx = blockIdx.x;
        by = blockIdx.y;
        bz = blockIdx.z;
        d = d1;
        zc = zc1;
        ctl = ctl1;
        partials = partials1;
        slot = block_slot();
        if (threadIdx.x == 0 && threadIdx.y == 0) publish_args(a1, tab, sc);
    }
    if (ctl->stop) return;
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = bx * OX + tx - 1;
    const int y = by * OY + ty - 1;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 1 && ty >= 1;
    const bool xf = (x == 0), xl = (x == nx - 1), yf = (y == 0), yl = (y == ny - 1);
    const int oc = ty * BX + tx;
    const int ox = ty * BX + max(tx - 1, 0), oy = max(ty - 1, 0) * BX + tx;
    const int col = min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const float tau = sc[0], lam = sc[1], ilt = sc[2];
    float pa = 0.f, pb = 0.f;

    if constexpr (!THREE) {
        const float p1 = __ldg(tab[0] + col), p2 = __ldg(tab[1] + col);
        const float q1 = __ldg(tab[3 + 0] + col), q2 = __ldg(tab[3 + 1] + col), q3 = __ldg(tab[3 + 2] + col);
        // the pixel's own U, U0 and V, issued with the rest before the barrier
        // (each pixel is written only by its own thread)
        const float uo = tab[12][col], u0 = __ldg(tab[13] + col);
        const float v1 = tab[9 + 0][col], v2 = tab[9 + 1][col];
        sm[0][0][oc] = p1;
        sm[0][1][oc] = p2;
        sm[0][2][oc] = q1;
        sm[0][3][oc] = q2;
        sm[0][4][oc] = q3;
        __syncthreads();
        if (o_pt) {
            // DivProjP_2D + newU (TGV_core.c:277-298, 300-306)
            const float dv = bwd(p1, sm[0][0][ox], xf, xl) + bwd(p2, sm[0][1][oy], yf, yl);
            const float un = (lam * (uo + tau * dv) + tau * u0) * ilt;
            const float ue = 2.0f * un - uo;
            tab[12][col] = ue;
            if (CHECK) {
                const float df = ue - uo;
                pa = df * df;
                pb = ue * ue;
            }
            // UpdV_2D + newV (TGV_core.c:308-345)
            const float d1 = bwd(q1, sm[0][2][ox], xf, xl) + bwd(q3, sm[0][4][oy], yf, yl);
            const float d2 = bwd(q3, sm[0][4][ox], xf, xl) + bwd(q2, sm[0][3][oy], yf, yl);
            tab[9 + 0][col] = 2.0f * (v1 + tau * (p1 + d1)) - v1;
            tab[9 + 1][col] = 2.0f * (v2 + tau * (p2 + d2)) - v2;
        }
    } else {
        const int z0 = bz * zc;
        const int z1 = min(z0 + zc, nz);
        const int sxy = (int)d.sxy;
        auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
        // z predecessors (plane k-1): P3, Q3, Q5, Q6
        const int om = at(z0 - 1);
        float zp3 = __ldg(tab[2] + om), zq3 = __ldg(tab[3 + 2] + om), zq5 = __ldg(tab[3 + 4] + om),
              zq6 = __ldg(tab[3 + 5] + om);
        // plane k: P1..3, Q1..6 (every thread); U, U0, V1..3 (updated voxels)
        float c[9], cu = 0.f, cu0 = 0.f, cv[3] = {0.f, 0.f, 0.f};
        auto load = [&](int k, float* pq, float& u, float& u0, float* vv) {
            const int o = at(k);
            for (int i = 0; i < 3; i++) pq[i] = __ldg(tab[i] + o);
            for (int i = 0; i < 6; i++) pq[3 + i] = __ldg(tab[3 + i] + o);
            if (o_pt) {
                u = tab[12][o];
                u0 = __ldg(tab[13] + o);
                for (int i = 0; i < 3; i++) vv[i] = tab[9 + i][o];
            }
        };
        load(z0, c, cu, cu0, cv);

        auto step = [&](auto par, int k) {
            constexpr int S = decltype(par)::value;
            float n[9], nu = 0.f, nu0 = 0.f, nv[3] = {0.f, 0.f, 0.f};
            if (k + 1 < z1) load(k + 1, n, nu, nu0, nv);
            // c[0..2] = P1..P3, c[3..8] = Q1..Q6
            sm[S][0][oc] = c[0];
            sm[S][1][oc] = c[1];
            sm[S][2][oc] = c[3];
            sm[S][3][oc] = c[4];
            sm[S][4][oc] = c[6];
            sm[S][5][oc] = c[7];
            sm[S][6][oc] = c[8];
            __syncthreads();
            if (o_pt) {
                const bool zf = (k == 0), zl = (k == nz - 1);
                // DivProjP_3D + newU3D (TGV_core.c:448-472, 548-554)
                float dv = bwd(c[0], sm[S][0][ox], xf, xl) + bwd(c[1], sm[S][1][oy], yf, yl);
                dv = dv + bwd(c[2], zp3, zf, zl);
                const float un = (lam * (cu + tau * dv) + tau * cu0) * ilt;
                const float ue = 2.0f * un - cu;
                const int o = k * sxy + col;
                tab[12][o] = ue;
                if (CHECK) {
                    const float df = ue - cu;
                    pa += df * df;
                    pb += ue * ue;
                }
                // UpdV_3D + newV (TGV_core.c:474-533, 558-568)
                const float q1 = bwd(c[3], sm[S][2][ox], xf, xl), q4x = bwd(c[6], sm[S][4][ox], xf, xl),
                            q5x = bwd(c[7], sm[S][5][ox], xf, xl);
                const float q2 = bwd(c[4], sm[S][3][oy], yf, yl), q4y = bwd(c[6], sm[S][4][oy], yf, yl),
                            q6y = bwd(c[8], sm[S][6][oy], yf, yl);
                const float q6z = bwd(c[8], zq6, zf, zl), q5z = bwd(c[7], zq5, zf, zl), q3 = bwd(c[5], zq3, zf, zl);
                const float d1 = q1 + q4y + q5z, d2 = q4x + q2 + q6z, d3 = q5x + q6y + q3;
                tab[9 + 0][o] = 2.0f * (cv[0] + tau * (c[0] + d1)) - cv[0];
                tab[9 + 1][o] = 2.0f * (cv[1] + tau * (c[1] + d2)) - cv[1];
                tab[9 + 2][o] = 2.0f * (cv[2] + tau * (c[2] + d3)) - cv[2];
            }
            zp3 = c[2];
            zq3 = c[5];
            zq5 = c[7];
            zq6 = c[8];
            for (int i = 0; i < 9; i++) c[i] = n[i];
            cu = nu;
            cu0 = nu0;
            for (int i = 0; i < 3; i++) cv[i] = nv[i];
        };
        int k = z0;
        for (; k + 1 < z1; k += 2) {
            step(Ic<0>{}, k);
            step(Ic<1>{}, k + 1);
        }
        if (k < z1) step(Ic<0>{}, k);
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, slot);
}

// The dual half-iteration (DualP + ProjP, DualQ + ProjQ; TGV_core.c:200-275
// in 2D, 351-446 in 3D) as a 2.5D streaming kernel.  Forward differences of U
// and V with "0 at the last index": a tile needs a halo of one voxel on its
// high x and y sides only (thread (tx, ty) on voxel (x0 + tx, y0 + ty), 31 x
// 15 voxels updated per CTA).  U and V of every thread go to shared memory for
// the x/y successors; the z successor is the next plane, which each thread
// holds in registers anyway (loaded one plane ahead).  P and Q are updated in
// place (each voxel reads only its own).  HBM traffic: read U, V, P, Q; write
// P, Q (88 B per voxel in 3D, 48 B in 2D).
template <bool THREE, bool BATCH>
__global__ void __launch_bounds__(NT, 2) k_tgv_dual_stream(TgvArgs a1, Dims d1, int zc1, const StopCtl* ctl1,
                                                           const TgvBatchVol* __restrict__ vols,
                                                           const int* __restrict__ tile_vol) {
    constexpr int NV = THREE ? 4 : 3;  // U, V1, V2 (, V3)
    __shared__ float sm[2][NV][BY * BX];
    __shared__ float* volatile tab[14];
    __shared__ float sc[3];
    __shared__ float sa[2];  // alpha1, alpha0
    int bx, by, bz, zc;
    Dims d;
    const StopCtl* ctl;
    if constexpr (BATCH) {
        const long long t = blockIdx.x;
        const TgvBatchVol& V = vols[tile_vol[t]];
        const long long lt = t - V.ptile_base;
        bx = (int)(lt % V.pgx);
        by = (int)((lt / V.pgx) % V.pgy);
        bz = (int)(lt / ((long long)V.pgx * V.pgy));
        d = V.d;
        zc = V.pzc;
        ctl = V.ctl;
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            publish_args(V.args, tab, sc);
            sa[0] = V.args.alpha1;
            sa[1] = V.args.alpha0;
        }
    } else {
        bx = blockIdx.x;
        by = blockIdx.y;
        bz = blockIdx.z;
        d = d1;
        zc = zc1;
        ctl = ctl1;
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            publish_args(a1, tab, sc);
            sa[0] = a1.alpha1;
            sa[1] = a1.alpha0;
        }
    }
    if (ctl->stop) return;
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = bx * OX + tx;
    const int y = by * OY + ty;
    const bool in_xy = (x < nx) && (y < ny);
    const bool o_pt = in_xy && tx < OX && ty < OY;
    const bool xe = (x == nx - 1), ye = (y == ny - 1);
    const int oc = ty * BX + tx;
    const int ox = ty * BX + min(tx + 1, BX - 1), oy = min(ty + 1, BY - 1) * BX + tx;
    const int col = min(y, ny - 1) * nx + min(x, nx - 1);
    const float sigma = sc[0];  // sigma == tau (TGV_core.c:54-55)
    const float alpha1 = sa[0], alpha0 = sa[1];

    if constexpr (!THREE) {
        const float u = __ldg(tab[12] + col), v1 = __ldg(tab[9] + col), v2 = __ldg(tab[10] + col);
        // the pixel's own P and Q, issued before the barrier (each pixel is
        // written only by its own thread)
        const float pold1 = tab[0][col], pold2 = tab[1][col];
        const float qold1 = tab[3][col], qold2 = tab[4][col], qold3 = tab[5][col];
        sm[0][0][oc] = u;
        sm[0][1][oc] = v1;
        sm[0][2][oc] = v2;
        __syncthreads();
        if (o_pt) {
            // DualP_2D + ProjP_2D (TGV_core.c:200-232)
            float p1 = pold1 + (xe ? sigma * (-v1) : sigma * ((sm[0][0][ox] - u) - v1));
            float p2 = pold2 + (ye ? sigma * (-v2) : sigma * ((sm[0][0][oy] - u) - v2));
            const float gp = sqrtf(p1 * p1 + p2 * p2) / alpha1;
            if (gp > 1.0f) {
                const float ig = __frcp_rn(gp);
                p1 *= ig;
                p2 *= ig;
            }
            tab[0][col] = p1;
            tab[1][col] = p2;
            // DualQ_2D + ProjQ_2D (TGV_core.c:234-275)
            float q1 = 0.f, q11 = 0.f, q2 = 0.f, q22 = 0.f;
            if (!xe) {
                q1 = sm[0][1][ox] - v1;
                q11 = sm[0][2][ox] - v2;
            }
            if (!ye) {
                q2 = sm[0][2][oy] - v2;
                q22 = sm[0][1][oy] - v1;
            }
            float Q1 = qold1 + sigma * q1;
            float Q2 = qold2 + sigma * q2;
            float Q3 = qold3 + sigma * (0.5f * (q11 + q22));
            float g = sqrtf(Q1 * Q1 + Q2 * Q2 + 2.0f * Q3 * Q3);
            g = g / alpha0;
            if (g > 1.0f) {
                const float ig = __frcp_rn(g);
                Q1 *= ig;
                Q2 *= ig;
                Q3 *= ig;
            }
            tab[3][col] = Q1;
            tab[4][col] = Q2;
            tab[5][col] = Q3;
        }
    } else {
        const int z0 = bz * zc;
        const int z1 = min(z0 + zc, nz);
        const int sxy = (int)d.sxy;
        auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
        auto ld_uv = [&](int k, float* w) {
            const int o = at(k);
            w[0] = __ldg(tab[12] + o);
            for (int i = 0; i < 3; i++) w[1 + i] = __ldg(tab[9 + i] + o);
        };
        float cw[4], nw[4];  // U, V1..V3 of planes k and k+1
        ld_uv(z0, cw);
        ld_uv(z0 + 1, nw);

        auto step = [&](auto par, int k) {
            constexpr int S = decltype(par)::value;
            float fw[4];  // plane k+2, used two steps on
            ld_uv(k + 2, fw);
            float pq[9];
            const int o = k * sxy + col;
            if (o_pt)
                for (int i = 0; i < 9; i++) pq[i] = tab[i][o];
            for (int i = 0; i < 4; i++) sm[S][i][oc] = cw[i];
            __syncthreads();
            if (o_pt) {
                const bool ze = (k == nz - 1);
                const float u = cw[0], v1 = cw[1], v2 = cw[2], v3 = cw[3];
                // DualP_3D + ProjP_3D (TGV_core.c:351-387)
                float p1 = pq[0] + (xe ? sigma * (-v1) : sigma * ((sm[S][0][ox] - u) - v1));
                float p2 = pq[1] + (ye ? sigma * (-v2) : sigma * ((sm[S][0][oy] - u) - v2));
                float p3 = pq[2] + (ze ? sigma * (-v3) : sigma * ((nw[0] - u) - v3));
                const float gp = sqrtf(p1 * p1 + p2 * p2 + p3 * p3) / alpha1;
                if (gp > 1.0f) {
                    const float ig = __frcp_rn(gp);
                    p1 *= ig;
                    p2 *= ig;
                    p3 *= ig;
                }
                tab[0][o] = p1;
                tab[1][o] = p2;
                tab[2][o] = p3;
                // DualQ_3D + ProjQ_3D (TGV_core.c:389-446)
                float q1 = 0.f, q11 = 0.f, q33 = 0.f, q2 = 0.f, q22 = 0.f, q55 = 0.f, q3 = 0.f, q44 = 0.f, q66 = 0.f;
                if (!xe) {
                    q1 = sm[S][1][ox] - v1;
                    q11 = sm[S][2][ox] - v2;
                    q33 = sm[S][3][ox] - v3;
                }
                if (!ye) {
                    q2 = sm[S][2][oy] - v2;
                    q22 = sm[S][1][oy] - v1;
                    q55 = sm[S][3][oy] - v3;
                }
                if (!ze) {
                    q3 = nw[3] - v3;
                    q44 = nw[1] - v1;
                    q66 = nw[2] - v2;
                }
                float Q1 = pq[3] + sigma * q1;
                float Q2 = pq[4] + sigma * q2;
                float Q3 = pq[5] + sigma * q3;
                float Q4 = pq[6] + sigma * (0.5f * (q11 + q22));
                float Q5 = pq[7] + sigma * (0.5f * (q33 + q44));
                float Q6 = pq[8] + sigma * (0.5f * (q55 + q66));
                float g = sqrtf(Q1 * Q1 + Q2 * Q2 + Q3 * Q3 + 2.0f * Q4 * Q4 + 2.0f * Q5 * Q5 + 2.0f * Q6 * Q6);
                g = g / alpha0;
                if (g > 1.0f) {
                    const float ig = __frcp_rn(g);
                    Q1 *= ig;
                    Q2 *= ig;
                    Q3 *= ig;
                    Q4 *= ig;
                    Q5 *= ig;
                    Q6 *= ig;
                }
                tab[3][o] = Q1;
                tab[4][o] = Q2;
                tab[5][o] = Q3;
                tab[6][o] = Q4;
                tab[7][o] = Q5;
                tab[8][o] = Q6;
            }
            for (int i = 0; i < 4; i++) {
                cw[i] = nw[i];
                nw[i] = fw[i];
            }
        };
        int k = z0;
        for (; k + 1 < z1; k += 2) {
            step(Ic<0>{}, k);
            step(Ic<1>{}, k + 1);
        }
        if (k < z1) step(Ic<0>{}, k);
    }
}

}  // namespace

TgvPlan tgv_primal_plan(const Dims& d) {
    TgvPlan T;
    const char* e = getenv("CILREG_TGV_KERNEL");
    // "simple" selects the per-voxel primal kernel; volumes of 2^31 voxels or
    // more use it too (this kernel indexes with 32-bit offsets)
    T.use = !(e && e[0] == 's') && d.n < (1LL << 31);
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_tgv_primal_stream<true, false, false>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 0, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int tgv_primal_stream_step(const TgvPlan& T, const TgvArgs& a, const Dims& d, const StopCtl* ctl, double2* partials,
                           cudaStream_t s) {
    const bool three = d.nz > 1;
    auto kern = three ? (a.check ? k_tgv_primal_stream<true, true, false> : k_tgv_primal_stream<true, false, false>)
                      : (a.check ? k_tgv_primal_stream<false, true, false> : k_tgv_primal_stream<false, false, false>);
    kern<<<T.grid, T.block, 0, s>>>(a, d, T.zchunk, ctl, partials, nullptr, nullptr);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int tgv_dual_stream_step(const TgvPlan& T, const TgvArgs& a, const Dims& d, const StopCtl* ctl, cudaStream_t s) {
    auto kern = (d.nz > 1) ? k_tgv_dual_stream<true, false> : k_tgv_dual_stream<false, false>;
    kern<<<T.grid, T.block, 0, s>>>(a, d, T.zchunk, ctl, nullptr, nullptr);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int tgv_dual_batch_step(const TgvBatchVol* d_vols, const int* d_ptile_vol, long long nptiles, bool three,
                        cudaStream_t s) {
    if (nptiles < 1 || nptiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", nptiles);
    auto kern = three ? k_tgv_dual_stream<true, true> : k_tgv_dual_stream<false, true>;
    TgvArgs none{};
    kern<<<dim3((unsigned)nptiles), dim3(BX, BY, 1), 0, s>>>(none, Dims{}, 1, nullptr, d_vols, d_ptile_vol);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

void tgv_primal_tiles(const Dims& d, int& gx, int& gy, int& gz, int& zc) {
    zc = (d.nz > 1) ? ((d.nz < ZCHUNK) ? d.nz : ZCHUNK) : 1;
    gx = (d.nx + OX - 1) / OX;
    gy = (d.ny + OY - 1) / OY;
    gz = (d.nz + zc - 1) / zc;
}

int tgv_primal_batch_step(const TgvBatchVol* d_vols, const int* d_ptile_vol, long long nptiles, bool three, int check,
                          cudaStream_t s) {
    if (nptiles < 1 || nptiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", nptiles);
    auto kern = three ? (check ? k_tgv_primal_stream<true, true, true> : k_tgv_primal_stream<true, false, true>)
                      : (check ? k_tgv_primal_stream<false, true, true> : k_tgv_primal_stream<false, false, true>);
    TgvArgs none{};
    kern<<<dim3((unsigned)nptiles), dim3(BX, BY, 1), 0, s>>>(none, Dims{}, 1, nullptr, nullptr, d_vols, d_ptile_vol);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace cilreg
