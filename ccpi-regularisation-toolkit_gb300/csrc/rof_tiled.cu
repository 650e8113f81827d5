// ROF-TV iteration as a 2.5D streaming stencil (2D images are the nz == 1 case).
//
// Reference arithmetic: ROF_TV_core.c:102-317.  Per voxel the update needs the
// three normalised fluxes D1 (j axis), D2 (i axis), D3 (k axis) at the voxel
// and at its mirrored lower neighbour on the same axis; each flux needs U on
// the 7-point mirrored neighbourhood.
//
// A CTA of 32 x 16 threads holds an overlapping tile: thread (tx, ty) sits on
// voxel (x0 - 2 + tx, y0 - 2 + ty); fluxes are formed on the inner 30 x 14
// voxels and the update on the inner 28 x 12.  Walking a chunk of z planes,
// step j of each thread:
//   A. forms the fluxes of plane j-1 once per voxel (three minmods, three
//      normalisations) from U of plane j-1 in shared memory (x/y
//      neighbours) and its own registers U(j-2), U(j) (z neighbours);
//      D1, D2 go to shared memory, D3 stays in a register;
//   B. publishes U(j) (prefetched one step earlier) to shared memory;
//   C. updates plane j-2: U += tau (lambda div D - (U - f)), with D3 of the
//      lower z neighbour from its own registers (plane 1 when j-2 == 0,
//      the mirror of ROF_TV_core.c:287).
// One barrier per plane; mirrored boundaries are neighbour-index selections.
// HBM traffic: read U and f, write U (12 B/voxel) plus the tile halo from L2.
#include "rof_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 4, OY = BY - 4;  // updated voxels per tile
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

// 0.5 (sign a + sign b) min(|a|, |b|) of ROF_TV_core.c:132, as sign-case selects
// (the same value: the smaller magnitude with the common sign, else 0)
__device__ __forceinline__ float minmod(float a, float b) {
    return (a > 0.f && b > 0.f) ? fminf(a, b) : ((a < 0.f && b < 0.f) ? fmaxf(a, b) : 0.f);
}

// dp / sqrt(s): one reciprocal square root instead of an IEEE square root and
// division (within 2 ulp of the reference's quotient)
__device__ __forceinline__ float normalise(float dp, float s) { return dp * rsqrtf(s); }

template <bool THREE>
__global__ void __launch_bounds__(NT, 3) k_rof_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                      const float* __restrict__ F, const float* __restrict__ lam_arr,
                                                      float lam, float tau, Dims d, int zc, const StopCtl* ctl,
                                                      int check, double2* partials) {
    __shared__ float sU[2][BY][BX];
    __shared__ float sD1[2][BY][BX];
    __shared__ float sD2[2][BY][BX];
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool d_pt = in_xy && tx >= 1 && tx <= BX - 2 && ty >= 1 && ty <= BY - 2;  // fluxes formed here
    const bool o_pt = in_xy && tx >= 2 && tx <= BX - 3 && ty >= 2 && ty <= BY - 3;  // update written here
    // mirrored neighbour columns/rows inside the tile (an axis of length 1 maps to itself)
    const int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    const int xl = (nx == 1) ? tx : ((x - 1 < 0) ? tx + 1 : tx - 1);
    const int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    const int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    const long long col = in_xy ? ((long long)y * nx + x) : 0;
    auto load_u = [&](int k) -> float {
        return (in_xy && k >= 0 && k < nz) ? __ldg(U + (long long)k * d.sxy + col) : 0.f;
    };

    // f (and lambda) of plane k, needed only where the update is written
    auto load_f = [&](int k, float& fv, float& lv) {
        fv = 0.f;
        lv = lam;
        if (o_pt && k >= z0 && k < z1) {
            const long long v = (long long)k * d.sxy + col;
            fv = __ldg(F + v);
            if (lam_arr) lv = __ldg(lam_arr + v);
        }
    };

    // register pipeline: U is loaded two planes before it is published, f two
    // planes before its update, so about two planes of loads are in flight
    float um2 = load_u(z0 - 2), um1 = load_u(z0 - 1);  // U(j-2), U(j-1) at step j = z0
    float uj = load_u(z0);                             // U(j)
    float uq = load_u(z0 + 1);                         // U(j+1)
    float fa, la, fb, lb;                              // f, lambda of planes j-2 and j-1
    load_f(z0 - 2, fa, la);
    load_f(z0 - 1, fb, lb);
    float d3a = 0.f, d3b = 0.f, d3c = 0.f;             // D3 of planes j-1, j-2, j-3
    float pa = 0.f, pb = 0.f;
    sU[(z0 - 1) & 1][ty][tx] = um1;
    __syncthreads();

    for (int j = z0; j <= z1 + 1; ++j) {
        const float un2 = (j + 2 <= z1) ? load_u(j + 2) : 0.f;  // prefetch U(j+2)
        float fn, ln;
        load_f(j, fn, ln);                                      // prefetch f(j)
        const int kf = j - 2;                                   // plane updated in step C
        const float fk = fa, lk = la;
        // A. fluxes of plane m = j-1
        const int m = j - 1;
        d3c = d3b;
        d3b = d3a;
        d3a = 0.f;
        if (m >= z0 - 1 && m >= 0 && m < nz && m <= z1 - 1) {
            const int sm = m & 1;
            if (d_pt) {
                const float c = sU[sm][ty][tx];
                const float xp = sU[sm][ty][xh] - c, xm = c - sU[sm][ty][xl];
                const float yp = sU[sm][yh][tx] - c, ym = c - sU[sm][yl][tx];
                const float mx = minmod(xp, xm), my = minmod(yp, ym);
                float d1, d2;
                if (THREE) {
                    const float zlo = (m == 0) ? uj : um2;          // mirrored lower plane
                    const float zhi = (m == nz - 1) ? um2 : uj;     // mirrored upper plane
                    const float zp = zhi - c, zm = c - zlo;
                    const float mz = minmod(zp, zm);
                    d1 = normalise(yp, yp * yp + mx * mx + mz * mz + 1.0e-8f);
                    d2 = normalise(xp, xp * xp + my * my + mz * mz + 1.0e-8f);
                    d3a = normalise(zp, zp * zp + my * my + mx * mx + 1.0e-8f);
                } else {
                    d1 = normalise(yp, yp * yp + mx * mx + 1.0e-8f);
                    d2 = normalise(xp, xp * xp + my * my + 1.0e-8f);
                }
                sD1[sm][ty][tx] = d1;
                sD2[sm][ty][tx] = d2;
            }
        }
        // B. publish U(j)
        sU[j & 1][ty][tx] = uj;
        // C. update plane kf = j-2 (fluxes of kf were published in the previous step)
        if (o_pt && kf >= z0 && kf < z1) {
            const int sk = kf & 1;
            const float dv1 = sD1[sk][ty][tx] - sD1[sk][yl][tx];
            const float dv2 = sD2[sk][ty][tx] - sD2[sk][ty][xl];
            float div;
            if (THREE) {
                const float d3lo = (kf == 0) ? d3a : d3c;  // D3 of the mirrored lower plane
                div = dv1 + dv2 + (d3b - d3lo);
            } else {
                div = dv1 + dv2;
            }
            const float u = um2;
            const float un = u + tau * (lk * div - (u - fk));
            Un[(long long)kf * d.sxy + col] = un;
            if (check) {
                const float df = un - u;
                pa += df * df;
                pb += un * un;
            }
        }
        __syncthreads();
        um2 = um1;
        um1 = uj;
        uj = uq;
        uq = un2;
        fa = fb;
        la = lb;
        fb = fn;
        lb = ln;
    }
    if (check) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

}  // namespace

RofPlan rof_tiled_plan(const Dims& d) {
    RofPlan T;
    T.zchunk = (d.nz > 1) ? ((d.nz < ZCHUNK) ? d.nz : ZCHUNK) : 1;
    T.block = dim3(BX, BY, 1);
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int rof_tiled_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                   float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    if (d.nz > 1)
        k_rof_stream<true><<<T.grid, T.block, 0, s>>>(cur, nxt, f, lam_arr, lam, tau, d, T.zchunk, ctl, check,
                                                      partials);
    else
        k_rof_stream<false><<<T.grid, T.block, 0, s>>>(cur, nxt, f, lam_arr, lam, tau, d, T.zchunk, ctl, check,
                                                       partials);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace cilreg
