// LLT-ROF: the fourth-order Lysaker-Lundervold-Tai term combined with ROF-TV
// in one explicit flow (reference: LLT_ROF_core.c:54-436):
//   U += tau (lambdaROF div D_ROF - lambdaLLT lap D_LLT - (U - f)),
// D_ROF the normalised ROF fluxes (minmod terms, eps 1e-12), D_LLT the
// per-axis second differences normalised by their magnitude,
// dxx / (|dxx| + 1e-12), all with mirrored boundaries.
//
// One 2.5D streaming kernel per iteration.  The update needs D_LLT at both
// neighbours on every axis, so a CTA of 32 x 16 threads holds a tile with a
// two-voxel halo (thread (tx, ty) on voxel (x0 - 2 + tx, y0 - 2 + ty)) and
// updates the inner 28 x 12.  Step j of each thread, walking a chunk of z:
//   B. publishes U(j) into a four-plane shared ring;
//   A. after the barrier, forms the ROF fluxes and the LLT terms of plane j-1
//      once per voxel; D1, D2 (ROF) and the x, y LLT terms go to shared
//      memory, the z terms stay in registers;
//   C. updates plane j-2 (terms summed in the reference's order).
// HBM traffic: read U and f, write U (12 B per voxel).  Two CTAs per SM at
// about 60 registers: limited to 40 registers for three, the 3D variants
// spill and run slower (1.25 -> 1.30 ms per 512^3 iteration).  Element offsets are
// 32-bit below 2^31 voxels, 64-bit from there.
#include <math.h>
#include <stdlib.h>

#include <type_traits>

#include "drivers.cuh"
#include "llt.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 4, OY = BY - 4;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

// square of minmod(a, b) (LLT_ROF_core.c:228): the median of a, b and 0
__device__ __forceinline__ float minmod_sq(float a, float b) {
    const float m = fmaxf(fminf(a, b), fminf(fmaxf(a, b), 0.f));
    return m * m;
}

// second difference normalised by its magnitude (LLT_ROF_core.c:148-152);
// the reference adds 1e-12 in double and stores the sum in a float, here the
// sum is formed in float (the same denominator within an ulp)
__device__ __forceinline__ float llt_term(float dxx) { return dxx / (fabsf(dxx) + 1.0e-12f); }

template <bool THREE, bool CHECK, class IT>
__global__ void __launch_bounds__(NT, 2) k_llt_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                      const float* __restrict__ F, float lam_rof, float lam_llt,
                                                      float tau, Dims d, int zc, const StopCtl* ctl,
                                                      double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU[4][BY * BX];
    __shared__ float sR1[2][BY * BX];  // ROF D1 (j axis), read at j-1
    __shared__ float sR2[2][BY * BX];  // ROF D2 (i axis), read at i-1
    __shared__ float sL1[2][BY * BX];  // LLT i term, read at i+-1
    __shared__ float sL2[2][BY * BX];  // LLT j term, read at j+-1
    if (ctl->stop) return;
    const float EPS = 1.0e-12f;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 2 && tx <= BX - 3 && ty >= 2 && ty <= BY - 3;
    // mirrored neighbours in the tile (an axis of length 1 maps to itself),
    // clamped to the tile where only unused halo values depend on them
    int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    int xl = (nx == 1) ? tx : ((x - 1 < 0) ? tx + 1 : tx - 1);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    xh = min(max(xh, 0), BX - 1);
    xl = min(max(xl, 0), BX - 1);
    yh = min(max(yh, 0), BY - 1);
    yl = min(max(yl, 0), BY - 1);
    const int oc = ty * BX + tx;
    const int oxh = ty * BX + xh, oxl = ty * BX + xl, oyh = yh * BX + tx, oyl = yl * BX + tx;
    const IT col = (IT)min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const IT sxy = (IT)d.sxy;
    auto at = [&](int k) -> IT { return (IT)min(max(k, 0), nz - 1) * sxy + col; };

    // z registers: ROF D3 and the LLT z term of planes j-1 (a), j-2 (b), j-3 (c)
    float r3a = 0.f, r3b = 0.f, r3c = 0.f, l3a = 0.f, l3b = 0.f, l3c = 0.f;
    float pa = 0.f, pb = 0.f;
    // U ring slot of plane p: (p - z0 + 4) & 3; flux slot: (p - z0 + 2) & 1
    sU[2][oc] = __ldg(U + at(z0 - 2));
    sU[3][oc] = __ldg(U + at(z0 - 1));
    float uj = __ldg(U + at(z0));
    float fa = o_pt ? __ldg(F + at(z0 - 2)) : 0.f, fb = o_pt ? __ldg(F + at(z0 - 1)) : 0.f;

    // steady steps (js0 <= j <= js1, 3D): every plane inside the volume and
    // the chunk and none the first or last plane of the volume, so no clamp,
    // no mirrored-plane select and no range test
    const int js0 = max(z0 + 2, 3), js1 = min(z1 + 1, nz - 2);
    auto step = [&](auto rr, auto st, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr bool ST = THREE && decltype(st)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // flux slots of planes j-1, j-2
        const float un1 = __ldg(U + (ST ? (IT)(j + 1) * sxy + col : at(j + 1)));  // prefetch U(j+1)
        const float fn = o_pt ? __ldg(F + (ST ? (IT)j * sxy + col : at(j))) : 0.f;  // prefetch f(j)
        // B. publish U(j)
        sU[SJ][oc] = uj;
        __syncthreads();
        // A. terms of plane m = j-1 (mirrored k neighbours)
        const int m = j - 1;
        {
            const float* Um = sU[SM];
            const float* Ulo = ST ? sU[SM2] : (THREE ? ((m == 0) ? sU[SJ] : sU[SM2]) : Um);
            const float* Uhi = ST ? sU[SJ] : (THREE ? ((m == nz - 1) ? sU[SM2] : sU[SJ]) : Um);
            const float c = Um[oc];
            const float xp = Um[oxh] - c, xm = c - Um[oxl];
            const float yp = Um[oyh] - c, ym = c - Um[oyl];
            const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym);
            float n1, n2, n3 = 0.f;
            if (THREE) {
                const float zp = Uhi[oc] - c, zm = c - Ulo[oc];
                const float mz2 = minmod_sq(zp, zm);
                n1 = yp * rsqrtf(yp * yp + mx2 + mz2 + EPS);
                n2 = xp * rsqrtf(xp * xp + my2 + mz2 + EPS);
                n3 = zp * rsqrtf(zp * zp + my2 + mx2 + EPS);
                l3c = l3b;
                l3b = l3a;
                l3a = llt_term(Uhi[oc] - 2.0f * c + Ulo[oc]);
            } else {
                n1 = yp * rsqrtf(yp * yp + mx2 + EPS);
                n2 = xp * rsqrtf(xp * xp + my2 + EPS);
            }
            r3c = r3b;
            r3b = r3a;
            r3a = n3;
            sR1[WM][oc] = n1;
            sR2[WM][oc] = n2;
            sL1[WM][oc] = llt_term(Um[oxh] - 2.0f * c + Um[oxl]);
            sL2[WM][oc] = llt_term(Um[oyh] - 2.0f * c + Um[oyl]);
        }
        // C. update plane kf = j-2 (its terms were published in the previous step)
        const int kf = j - 2;
        if (o_pt && (ST || (kf >= z0 && kf < z1))) {
            const float w1 = sL1[WK][oc], w2 = sL2[WK][oc];
            const float dxx = sL1[WK][oxh] - 2.0f * w1 + sL1[WK][oxl];
            const float dyy = sL2[WK][oyh] - 2.0f * w2 + sL2[WK][oyl];
            const float dv1 = sR1[WK][oc] - sR1[WK][oyl];
            const float dv2 = sR2[WK][oc] - sR2[WK][oxl];
            float laplc, div;
            if (THREE) {
                const float llo = (!ST && kf == 0) ? l3a : l3c;        // mirrored k-1
                const float lhi = (!ST && kf == nz - 1) ? l3c : l3a;   // mirrored k+1
                const float dzz = lhi - 2.0f * l3b + llo;
                laplc = dxx + dyy + dzz;
                const float rlo = (!ST && kf == 0) ? r3a : r3c;
                div = dv1 + dv2 + (r3b - rlo);
            } else {
                laplc = dxx + dyy;
                div = dv1 + dv2;
            }
            const float u = sU[SM2][oc];
            const float un = u + tau * (lam_rof * div - lam_llt * laplc - (u - fa));
            Un[(IT)kf * sxy + col] = un;
            if (CHECK) {
                const float df = un - u;
                pa += df * df;
                pb += un * un;
            }
        }
        uj = un1;
        fa = fb;
        fb = fn;
    };
    // each position of the unrolled loop runs the steady or the general step
    // (a branch on the plane index, the same for the whole CTA)
    auto any = [&](auto rr, int jj) {
        if (jj >= js0 && jj <= js1) step(rr, std::true_type{}, jj);
        else step(rr, std::false_type{}, jj);
    };
    int j = z0;
    for (; j + 3 <= z1 + 1; j += 4) {
        any(Ic<0>{}, j);
        any(Ic<1>{}, j + 1);
        any(Ic<2>{}, j + 2);
        any(Ic<3>{}, j + 3);
    }
    if (j <= z1 + 1) step(Ic<0>{}, std::false_type{}, j);
    if (j + 1 <= z1 + 1) step(Ic<1>{}, std::false_type{}, j + 1);
    if (j + 2 <= z1 + 1) step(Ic<2>{}, std::false_type{}, j + 2);
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

LltPlan llt_plan(const Dims& d) {
    if (llt_pair_applies(d)) return llt_pair_plan(d);
    LltPlan T;
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_llt_stream<true, false, int>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

}  // namespace

int llt_run(const float* f, float* u_out, float lam_rof, float lam_llt, int iters, float tau, float epsil,
            const Dims& d, cudaStream_t s, float* info) {
    CILREG_RANGE("cilreg LLT-ROF");
    Scratch scratch(s);
    const LltPlan T = llt_plan(d);
    IterControl ctl(s, scratch, iters, epsil, T.nblocks);
    CILREG_TRY(ctl.status());
    float* alt = scratch.floats(d.n);
    if (!alt) return scratch.status();
    float* bufs[2] = {u_out, alt};
    CILREG_CUDA(cudaMemcpyAsync(u_out, f, sizeof(float) * d.n, cudaMemcpyDeviceToDevice, s));
    const bool three = d.nz > 1;
    auto launch = [&](const float* cur, float* nxt, int check, cudaStream_t st) -> cudaError_t {
        if (T.pair)
            return llt_pair_launch(T, cur, nxt, f, lam_rof, lam_llt, tau, d, ctl.ctl(), check, ctl.partials(), st);
        decltype(&k_llt_stream<true, true, int>) kern;
        if (d.n < (1LL << 31))
            kern = three ? (check ? k_llt_stream<true, true, int> : k_llt_stream<true, false, int>)
                         : (check ? k_llt_stream<false, true, int> : k_llt_stream<false, false, int>);
        else
            kern = three ? (check ? k_llt_stream<true, true, long long> : k_llt_stream<true, false, long long>)
                         : (check ? k_llt_stream<false, true, long long> : k_llt_stream<false, false, long long>);
        return launch_pdl(kern, T.grid, T.block, 0, st, cur, nxt, f, lam_rof, lam_llt, tau, d, T.zchunk,
                          (const StopCtl*)ctl.ctl(), ctl.partials());
    };
    int it = 0;
    if (!ctl.checking() && d.n <= (1LL << 22)) {
        // small volume, fixed count: launch overhead dominates, replay a graph
        CILREG_TRY(run_replayed(iters, 64, s, [&](int k, cudaStream_t st, bool) -> int {
            CILREG_CUDA(launch(bufs[k & 1], bufs[(k + 1) & 1], 0, st));
            note_launch();
            return OK;
        }));
        it = iters;
    }
    for (; it < iters; it++) {
        const int check = ctl.is_check(it) ? 1 : 0;
        CILREG_CUDA(launch(bufs[it & 1], bufs[(it + 1) & 1], check, s));
        note_launch();
        if (check) {
            CILREG_TRY(ctl.after_check(it, T.nblocks));
            if (ctl.host_should_stop()) break;
        }
    }
    if (iters > 0) CILREG_TRY(launch_select_pingpong(ctl.ctl(), iters, bufs, u_out, d.n, s));
    return ctl.finish(info);
}

}  // namespace cilreg
