// ROF-TV iteration as a 2.5D streaming stencil (2D images are the nz == 1 case).
//
// Reference arithmetic: ROF_TV_core.c:102-317.  Per voxel the update needs the
// three normalised fluxes D1 (j axis), D2 (i axis), D3 (k axis) at the voxel
// and at its mirrored lower neighbour on the same axis.  D1 needs U at the
// voxel, its upper j neighbour and both i neighbours (minmod); D2 the mirror
// image of that; so the update of a voxel reads U only within one voxel of it
// in i and j, and the lower-neighbour fluxes D1(j-1), D2(i-1) need no U beyond
// that either.
//
// A CTA of 32 x 16 threads holds an overlapping tile with a one-voxel halo:
// thread (tx, ty) sits on voxel (x0 - 1 + tx, y0 - 1 + ty) and the inner
// 30 x 14 voxels are updated.  Walking a chunk of z planes, step j of each
// thread:
//   A. forms the fluxes of plane j-1 (three minmods, three normalisations)
//      from U of plane j-1 in shared memory (i/j neighbours) and its own
//      registers U(j-2), U(j) (k neighbours); D1, D2 go to shared memory, all
//      three stay in registers for the thread's own update;
//   B. publishes U(j) (loaded two steps earlier) to shared memory;
//   C. updates plane j-2: U += tau (lambda div D - (U - f)).
// One barrier per plane.  The i/j mirrors are per-thread neighbour offsets
// and the k mirror two selects on the plane index, so the steady loop has no
// boundary branches; shared-memory ring slots are compile-time constants
// (the loop is unrolled by two).  The z chunk length balances the CTAs over
// the SMs (wave_zchunk).  HBM traffic: read U and f, write U
// (12 B/voxel) plus the tile halo from L2.
#include <stdlib.h>

#include <type_traits>

#include "rof_tiled.cuh"
#include "tma_ring.cuh"

namespace cilreg {

namespace {

using tma::cp_async4;
using tma::cp_async_commit;
using tma::cp_async_wait;

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 2, OY = BY - 2;  // updated voxels per tile
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

// square of minmod(a, b) = 0.5 (sign a + sign b) min(|a|, |b|)
// (ROF_TV_core.c:132): the median of a, b and 0 has the same magnitude
__device__ __forceinline__ float minmod_sq(float a, float b) {
    const float m = fmaxf(fminf(a, b), fminf(fmaxf(a, b), 0.f));
    return m * m;
}

// dp / sqrt(s): one reciprocal square root instead of an IEEE square root and
// division (within 2 ulp of the reference's quotient)
__device__ __forceinline__ float normalise(float dp, float s) { return dp * rsqrtf(s); }

template <int V>
using Ic = std::integral_constant<int, V>;

// the value of an integral constant or of a plain int, on the device
template <int V>
__device__ __forceinline__ constexpr int ival(Ic<V>) {
    return V;
}
__device__ __forceinline__ int ival(int v) { return v; }

// IT: element-offset type (int when the volume has fewer than 2^31 voxels)
template <bool THREE, bool CHECK, bool LARR, typename IT>
__global__ void __launch_bounds__(NT, 3) k_rof_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                      const float* __restrict__ F, const float* __restrict__ lam_arr,
                                                      float lam, float tau, Dims d, int zc, const StopCtl* ctl,
                                                      double2* partials) {
    __shared__ float sU[2][BY * BX];
    __shared__ float sD1[2][BY * BX];
    __shared__ float sD2[2][BY * BX];
    const float EPS = 1.0e-8f;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 1;
    const int y = blockIdx.y * OY + ty - 1;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 1 && tx <= BX - 2 && ty >= 1 && ty <= BY - 2;
    // neighbour columns / rows in the tile: mirrored at the volume edge (an axis
    // of length 1 maps to itself), clamped to the tile elsewhere (a clamped
    // neighbour only feeds fluxes that no update reads)
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
    // halo threads outside the volume load the nearest voxel inside it (their
    // fluxes are never read), so loads need no predicate
    const IT col = (IT)min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    float pa = 0.f, pb = 0.f;
    // f and the lambda map never change during a run: in a plane they are
    // loaded before waiting for the previous iteration (launch_pdl)
    float fv0 = 0.f, lv0 = lam;
    if constexpr (!THREE) {
        fv0 = o_pt ? __ldg(F + col) : 0.f;
        lv0 = (LARR && o_pt) ? __ldg(lam_arr + col) : lam;
    }
    pdl_wait();  // the previous iteration has completed and its writes are visible
    pdl_trigger();
    if (ctl->stop) return;

    if constexpr (!THREE) {
        // one plane: publish U, form D1/D2, update
        const float u = __ldg(U + col);
        const float fv = fv0;
        const float lv = lv0;
        sU[0][oc] = u;
        __syncthreads();
        const float xp = sU[0][oxh] - u, xm = u - sU[0][oxl];
        const float yp = sU[0][oyh] - u, ym = u - sU[0][oyl];
        const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym);
        const float d1 = normalise(yp, yp * yp + mx2 + EPS);
        const float d2 = normalise(xp, xp * xp + my2 + EPS);
        sD1[0][oc] = d1;
        sD2[0][oc] = d2;
        __syncthreads();
        if (o_pt) {
            const float div = (d1 - sD1[0][oyl]) + (d2 - sD2[0][oxl]);
            const float un = u + tau * (lv * div - (u - fv));
            Un[col] = un;
            if (CHECK) {
                const float df = un - u;
                pa = df * df;
                pb = un * un;
            }
        }
    } else {
        const int z0 = blockIdx.z * zc;
        const int z1 = min(z0 + zc, nz);
        const IT sxy = (IT)d.sxy;
        // element offset of plane k (clamped into the volume: planes outside it
        // are loaded only into pipeline slots that are never used unmirrored)
        auto at = [&](int k) -> IT { return (IT)min(max(k, 0), nz - 1) * sxy + col; };
        auto ld_u = [&](int k) -> float { return __ldg(U + at(k)); };
        auto ld_f = [&](int k, float& fv, float& lv) {
            const IT o = at(k);
            fv = o_pt ? __ldg(F + o) : 0.f;
            lv = (LARR && o_pt) ? __ldg(lam_arr + o) : lam;
        };
        // registers entering step j: U(j-2), U(j-1), U(j), U(j+1); f and lambda of
        // planes j-2, j-1; own fluxes of plane j-2 and D3 of plane j-3
        float ua = ld_u(z0 - 2), ub = ld_u(z0 - 1), uc = ld_u(z0), ud = ld_u(z0 + 1);
        float fa = 0.f, la = lam, fb = 0.f, lb = lam;
        float d1o = 0.f, d2o = 0.f, d3o = 0.f, d3oo = 0.f;
        sU[1][oc] = ub;  // ring slot of plane p: (p - z0) & 1
        __syncthreads();

        auto step = [&](auto par, auto full, int j) {
            constexpr int P = decltype(par)::value;    // ring slot of plane j
            constexpr bool FULL = decltype(full)::value;  // plane j-2 is updated
            const float ue = ld_u(j + 2);
            float fe, le;
            ld_f(j, fe, le);  // f, lambda of plane j (its update is two steps on)
            // A. fluxes of plane m = j-1 (ROF_TV_core.c:102-266); k neighbours
            // mirrored at the first and last plane (ROF_TV_core.c:117-118)
            const int m = j - 1;
            const float zlo = (m == 0) ? uc : ua;
            const float zhi = (m == nz - 1) ? ua : uc;
            const float xp = sU[1 - P][oxh] - ub, xm = ub - sU[1 - P][oxl];
            const float yp = sU[1 - P][oyh] - ub, ym = ub - sU[1 - P][oyl];
            const float zp = zhi - ub, zm = ub - zlo;
            const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym), mz2 = minmod_sq(zp, zm);
            const float n1 = normalise(yp, yp * yp + mx2 + mz2 + EPS);
            const float n2 = normalise(xp, xp * xp + my2 + mz2 + EPS);
            const float n3 = normalise(zp, zp * zp + my2 + mx2 + EPS);
            sD1[1 - P][oc] = n1;
            sD2[1 - P][oc] = n2;
            // B. publish U(j)
            sU[P][oc] = uc;
            // C. update plane j-2 (ROF_TV_core.c:269-297); its fluxes were
            // published in the previous step, the lower k flux is D3 of plane
            // j-3, mirrored to plane 1 at the first plane
            if (FULL) {
                const int kf = j - 2;
                const float d3lo = (kf == 0) ? n3 : d3oo;
                const float div = (d1o - sD1[P][oyl]) + (d2o - sD2[P][oxl]) + (d3o - d3lo);
                const float un = ua + tau * (la * div - (ua - fa));
                if (o_pt) Un[(IT)kf * sxy + col] = un;
                if (CHECK && o_pt) {
                    const float df = un - ua;
                    pa += df * df;
                    pb += un * un;
                }
            }
            __syncthreads();
            ua = ub;
            ub = uc;
            uc = ud;
            ud = ue;
            fa = fb;
            la = lb;
            fb = fe;
            lb = le;
            d3oo = d3o;
            d1o = n1;
            d2o = n2;
            d3o = n3;
        };
        step(Ic<0>{}, std::false_type{}, z0);
        step(Ic<1>{}, std::false_type{}, z0 + 1);
        int j = z0 + 2;
        for (; j + 1 <= z1 + 1; j += 2) {
            step(Ic<0>{}, std::true_type{}, j);
            step(Ic<1>{}, std::true_type{}, j + 1);
        }
        if (j <= z1 + 1) step(Ic<0>{}, std::true_type{}, j);
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// The 3D iteration with U staged through shared memory by asynchronous copies
// issued AHEAD planes early into an 8-plane ring, so that load latency is not
// bound to registers: step j issues plane j+AHEAD, waits for its own copy of
// plane j, and one barrier makes plane j (and the fluxes of plane j-2) visible
// to the CTA; then it forms the fluxes of plane j-1 and updates plane j-2 as
// k_rof_stream does.  Same arithmetic, same tile.
constexpr int AHEAD = 4;
constexpr int RING = 8;

template <bool CHECK, bool LARR, typename IT>
__global__ void __launch_bounds__(NT, 3) k_rof_async(const float* __restrict__ U, float* __restrict__ Un,
                                                     const float* __restrict__ F, const float* __restrict__ lam_arr,
                                                     float lam, float tau, Dims d, int zc, const StopCtl* ctl,
                                                     double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU[RING][BY * BX];
    __shared__ float sD1[2][BY * BX];
    __shared__ float sD2[2][BY * BX];
    if (ctl->stop) return;
    const float EPS = 1.0e-8f;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 1;
    const int y = blockIdx.y * OY + ty - 1;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 1 && tx <= BX - 2 && ty >= 1 && ty <= BY - 2;
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
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const IT sxy = (IT)d.sxy;
    auto at = [&](int k) -> IT { return (IT)min(max(k, 0), nz - 1) * sxy + col; };
    // ring slot of plane z0 + r - 2 (plane k sits in slot (k - z0 + 2) & 7)
    auto slot_of = [&](int r) -> float* { return sU[r & (RING - 1)]; };
    auto ld_f = [&](int k, float& fv, float& lv) {
        const IT o = at(k);
        fv = o_pt ? __ldg(F + o) : 0.f;
        lv = (LARR && o_pt) ? __ldg(lam_arr + o) : lam;
    };
    float pa = 0.f, pb = 0.f;
    // planes z0-2 .. z0+AHEAD-1 in flight, one copy group per plane
    for (int k = z0 - 2; k < z0 + AHEAD; k++) {
        cp_async4(slot_of(k - z0 + 2) + oc, U + at(k));
        cp_async_commit();
    }
    float fa = 0.f, la = lam, fb = 0.f, lb = lam;
    float d1o = 0.f, d2o = 0.f, d3o = 0.f, d3oo = 0.f;

    // step j, r = j - z0: an integral constant in the unrolled loop (every
    // ring slot and the flux parity fold to constants), a plain int in the
    // remainder
    auto step = [&](auto rr, auto full, int j) {
        const int r = ival(rr);
        const int P = r & 1;                          // flux ring slot of plane j
        constexpr bool FULL = decltype(full)::value;  // plane j-2 is updated
        cp_async4(slot_of(r + 2 + AHEAD) + oc, U + at(j + AHEAD));
        cp_async_commit();
        float fe, le;
        ld_f(j, fe, le);
        cp_async_wait<AHEAD>();  // this thread's copy of plane j has landed
        __syncthreads();         // ... and every thread's, and the fluxes of plane j-2
        const float* Uj = slot_of(r + 2);
        const float* Um = slot_of(r + 1);
        const float* Ua = slot_of(r);
        const float ub = Um[oc], uc = Uj[oc], ua = Ua[oc];
        // A. fluxes of plane m = j-1
        const int m = j - 1;
        const float zlo = (m == 0) ? uc : ua;
        const float zhi = (m == nz - 1) ? ua : uc;
        const float xp = Um[oxh] - ub, xm = ub - Um[oxl];
        const float yp = Um[oyh] - ub, ym = ub - Um[oyl];
        const float zp = zhi - ub, zm = ub - zlo;
        const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym), mz2 = minmod_sq(zp, zm);
        const float n1 = normalise(yp, yp * yp + mx2 + mz2 + EPS);
        const float n2 = normalise(xp, xp * xp + my2 + mz2 + EPS);
        const float n3 = normalise(zp, zp * zp + my2 + mx2 + EPS);
        sD1[1 - P][oc] = n1;
        sD2[1 - P][oc] = n2;
        // C. update plane j-2
        if (FULL) {
            const int kf = j - 2;
            const float d3lo = (kf == 0) ? n3 : d3oo;
            const float div = (d1o - sD1[P][oyl]) + (d2o - sD2[P][oxl]) + (d3o - d3lo);
            const float un = ua + tau * (la * div - (ua - fa));
            if (o_pt) Un[(IT)kf * sxy + col] = un;
            if (CHECK && o_pt) {
                const float df = un - ua;
                pa += df * df;
                pb += un * un;
            }
        }
        fa = fb;
        la = lb;
        fb = fe;
        lb = le;
        d3oo = d3o;
        d1o = n1;
        d2o = n2;
        d3o = n3;
    };
    step(Ic<0>{}, std::false_type{}, z0);
    step(Ic<1>{}, std::false_type{}, z0 + 1);
    int j = z0 + 2;
    for (; j + 7 <= z1 + 1; j += 8) {
        step(Ic<2>{}, std::true_type{}, j);
        step(Ic<3>{}, std::true_type{}, j + 1);
        step(Ic<4>{}, std::true_type{}, j + 2);
        step(Ic<5>{}, std::true_type{}, j + 3);
        step(Ic<6>{}, std::true_type{}, j + 4);
        step(Ic<7>{}, std::true_type{}, j + 5);
        step(Ic<8>{}, std::true_type{}, j + 6);
        step(Ic<9>{}, std::true_type{}, j + 7);
    }
    for (; j <= z1 + 1; j++) step(j - z0, std::true_type{}, j);
    cp_async_wait<0>();
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// ---------------------------------------------------------------------------
// 2D images, fixed iteration counts: `depth` iterations per launch on tiles
// with overlapped halos (ghost zones).  A CTA loads its 48 x 32 output tile
// plus `depth` pixels on every side (clipped at the image edge) of U and f
// (and the lambda map) into shared memory and runs `depth` iterations there:
// iteration t forms the fluxes on the region less t pixels on each side cut
// by the halo and updates it less t + 1, so after `depth` iterations the
// output tile holds U^(k+depth) exactly (a voxel's update reads U only within
// one pixel of it, diagonals included).  Neighbours outside the valid region
// are clamped into the region; what they feed lies outside the valid region
// and is never written out.  The per-pixel arithmetic is that of the 2D path
// of k_rof_stream.  One launch replaces `depth` launches, and U makes one
// round trip through L2/DRAM per `depth` iterations.
constexpr int TBW = 48, TBH = 32;   // output tile
constexpr int TBMAXD = 8;           // largest depth
constexpr int TBRW = TBW + 2 * TBMAXD, TBRH = TBH + 2 * TBMAXD;
constexpr int TBTX = 32, TBTY = 16;
constexpr int TBARR = TBRW * TBRH;

template <bool LARR>
__global__ void __launch_bounds__(TBTX * TBTY, 2) k_rof_tb2d(const float* __restrict__ U, float* __restrict__ Un,
                                                              const float* __restrict__ F,
                                                              const float* __restrict__ lam_arr, float lam,
                                                              float tau, Dims d, int depth) {
    extern __shared__ float smem[];
    float* sA = smem;
    float* sB = sA + TBARR;
    float* sD1 = sB + TBARR;
    float* sD2 = sD1 + TBARR;
    float* sF = sD2 + TBARR;
    float* sL = sF + TBARR;  // lambda map (LARR only)
    const float EPS = 1.0e-8f;
    const int nx = d.nx, ny = d.ny;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int ox0 = blockIdx.x * TBW, oy0 = blockIdx.y * TBH;
    const int rx0 = max(ox0 - depth, 0), ry0 = max(oy0 - depth, 0);
    const int rx1 = min(ox0 + TBW + depth, nx), ry1 = min(oy0 + TBH + depth, ny);
    const int rw = rx1 - rx0, rh = ry1 - ry0;
    const bool cutL = rx0 > 0, cutR = rx1 < nx, cutT = ry0 > 0, cutB = ry1 < ny;
    // f and the lambda map never change during a run: loaded before waiting
    // for the previous launch (launch_pdl)
    for (int y = ty; y < rh; y += TBTY)
        for (int x = tx; x < rw; x += TBTX) {
            const int g = (ry0 + y) * nx + rx0 + x;
            sF[y * TBRW + x] = __ldg(F + g);
            if (LARR) sL[y * TBRW + x] = __ldg(lam_arr + g);
        }
    pdl_wait();
    pdl_trigger();
    for (int y = ty; y < rh; y += TBTY)
        for (int x = tx; x < rw; x += TBTX) sA[y * TBRW + x] = __ldg(U + (ry0 + y) * nx + rx0 + x);
    __syncthreads();
    // mirrored neighbours in region coordinates (an axis of length 1 maps to
    // itself; a neighbour beyond a side cut by the halo is clamped)
    auto hi_x = [&](int x) { return (nx == 1) ? x : ((rx0 + x + 1 >= nx) ? x - 1 : min(x + 1, rw - 1)); };
    auto lo_x = [&](int x) { return (nx == 1) ? x : ((rx0 + x - 1 < 0) ? x + 1 : max(x - 1, 0)); };
    auto hi_y = [&](int y) { return (ny == 1) ? y : ((ry0 + y + 1 >= ny) ? y - 1 : min(y + 1, rh - 1)); };
    auto lo_y = [&](int y) { return (ny == 1) ? y : ((ry0 + y - 1 < 0) ? y + 1 : max(y - 1, 0)); };
    float* cur = sA;
    float* nxt = sB;
    for (int t = 0; t < depth; t++) {
        const int fx0 = cutL ? t : 0, fx1 = cutR ? rw - t : rw;
        const int fy0 = cutT ? t : 0, fy1 = cutB ? rh - t : rh;
        for (int y = fy0 + ty; y < fy1; y += TBTY) {
            const int yh = hi_y(y), yl = lo_y(y);
            for (int x = fx0 + tx; x < fx1; x += TBTX) {
                const float u = cur[y * TBRW + x];
                const float xp = cur[y * TBRW + hi_x(x)] - u, xm = u - cur[y * TBRW + lo_x(x)];
                const float yp = cur[yh * TBRW + x] - u, ym = u - cur[yl * TBRW + x];
                const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym);
                sD1[y * TBRW + x] = normalise(yp, yp * yp + mx2 + EPS);
                sD2[y * TBRW + x] = normalise(xp, xp * xp + my2 + EPS);
            }
        }
        __syncthreads();
        const int ux0 = cutL ? t + 1 : 0, ux1 = cutR ? rw - t - 1 : rw;
        const int uy0 = cutT ? t + 1 : 0, uy1 = cutB ? rh - t - 1 : rh;
        for (int y = uy0 + ty; y < uy1; y += TBTY) {
            const int yl = lo_y(y);
            for (int x = ux0 + tx; x < ux1; x += TBTX) {
                const int o = y * TBRW + x;
                const float u = cur[o];
                const float fv = sF[o];
                const float lv = LARR ? sL[o] : lam;
                const float div = (sD1[o] - sD1[yl * TBRW + x]) + (sD2[o] - sD2[y * TBRW + lo_x(x)]);
                nxt[o] = u + tau * (lv * div - (u - fv));
            }
        }
        __syncthreads();
        float* tmp = cur;
        cur = nxt;
        nxt = tmp;
    }
    // the output tile (clipped at the image edge)
    const int ty0 = oy0 - ry0, ty1 = min(oy0 + TBH, ny) - ry0;
    const int tx0 = ox0 - rx0, tx1 = min(ox0 + TBW, nx) - rx0;
    for (int y = ty0 + ty; y < ty1; y += TBTY)
        for (int x = tx0 + tx; x < tx1; x += TBTX) Un[(ry0 + y) * nx + rx0 + x] = cur[y * TBRW + x];
}

size_t tb2d_smem(bool larr) { return sizeof(float) * TBARR * (larr ? 6 : 5); }

template <bool LARR>
bool tb2d_smem_ok() {
    static const bool ok = [] {
        const bool r = cudaFuncSetAttribute(k_rof_tb2d<LARR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)tb2d_smem(LARR)) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    return ok;
}

}  // namespace

int rof_tb2d_depth(const Dims& d, int iters) {
    // opt-in: CILREG_ROF_TB=<depth> (1..8).  On a 512^2 image it ran 3.27 us
    // per iteration at depth 8 against 2.76 us for one launch per iteration
    // replayed from a graph: such a run is bound by the latency of an
    // iteration on about 1,700 pixels per SM, not by its launches.
    const char* e = getenv("CILREG_ROF_TB");
    if (d.nz != 1 || d.n >= (1LL << 31) || iters < 2 || !e || atoi(e) <= 0) return 0;
    return atoi(e) < TBMAXD ? atoi(e) : TBMAXD;
}

int rof_tb2d_step(const float* cur, float* nxt, const float* f, const float* lam_arr, float lam, float tau,
                  const Dims& d, int depth, cudaStream_t s) {
    if (depth < 1 || depth > TBMAXD) return fail(ERR_ARG, __FILE__, __LINE__, "depth %d out of range", depth);
    const bool larr = lam_arr != nullptr;
    if (!(larr ? tb2d_smem_ok<true>() : tb2d_smem_ok<false>()))
        return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_rof_tb2d");
    const dim3 grid((d.nx + TBW - 1) / TBW, (d.ny + TBH - 1) / TBH, 1), block(TBTX, TBTY, 1);
    if (larr)
        CILREG_CUDA(launch_pdl(k_rof_tb2d<true>, grid, block, tb2d_smem(true), s, cur, nxt, f, lam_arr, lam, tau, d,
                               depth));
    else
        CILREG_CUDA(launch_pdl(k_rof_tb2d<false>, grid, block, tb2d_smem(false), s, cur, nxt, f, lam_arr, lam, tau,
                               d, depth));
    return OK;
}

RofPlan rof_tiled_plan(const Dims& d) {
    if (rof_pair_applies(d)) return rof_pair_plan(d);
    RofPlan T;
    T.block = dim3(BX, BY, 1);
    const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
    if (d.nz > 1) {
        // CTAs per SM of the 3D kernel (every variant has the same register cap)
        static const int resident = resident_ctas(k_rof_stream<true, false, false, int>, NT);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int rof_tiled_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                   float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    if (T.pair) return rof_pair_step(T, cur, nxt, f, lam_arr, lam, tau, d, ctl, check, partials, s);
    const bool three = d.nz > 1, larr = lam_arr != nullptr;
    const char* ek = getenv("CILREG_ROF_KERNEL");
    if (three && d.n < (1LL << 31) && !(ek && ek[0] == 'r')) {
        // CILREG_ROF_KERNEL=reg keeps the register-pipelined kernel (A/B checks)
        auto ka = check ? (larr ? k_rof_async<true, true, int> : k_rof_async<true, false, int>)
                        : (larr ? k_rof_async<false, true, int> : k_rof_async<false, false, int>);
        CILREG_CUDA(launch_pdl(ka, T.grid, T.block, 0, s, cur, nxt, f, lam_arr, lam, tau, d, T.zchunk, ctl, partials));
        return OK;
    }
    decltype(&k_rof_stream<true, true, true, int>) kern;
    if (d.n < (1LL << 31)) {
        kern = three ? (check ? (larr ? k_rof_stream<true, true, true, int> : k_rof_stream<true, true, false, int>)
                              : (larr ? k_rof_stream<true, false, true, int> : k_rof_stream<true, false, false, int>))
                     : (check ? (larr ? k_rof_stream<false, true, true, int> : k_rof_stream<false, true, false, int>)
                              : (larr ? k_rof_stream<false, false, true, int> : k_rof_stream<false, false, false, int>));
    } else {
        kern = three ? (check ? (larr ? k_rof_stream<true, true, true, long long> : k_rof_stream<true, true, false, long long>)
                              : (larr ? k_rof_stream<true, false, true, long long> : k_rof_stream<true, false, false, long long>))
                     : (check ? (larr ? k_rof_stream<false, true, true, long long> : k_rof_stream<false, true, false, long long>)
                              : (larr ? k_rof_stream<false, false, true, long long> : k_rof_stream<false, false, false, long long>));
    }
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, cur, nxt, f, lam_arr, lam, tau, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
