// The two Jacobi sweeps of a split-Bregman outer iteration (reference:
// SB_TV_core.c:149-173 in 2D, 254-282 in 3D, called twice at :63-67 and
// :110-114) as one 2.5D streaming kernel with temporal depth two:
//   U1 = sweep(U0, D, B, f),  U2 = sweep(U1, D, B, f).
// D and B are the same in both sweeps, so their divergence term G is formed
// once per voxel.  U1 never reaches memory.
//
// A CTA of 32 x 16 threads holds a tile with a two-voxel halo: thread (tx, ty)
// on voxel (x0 - 2 + tx, y0 - 2 + ty).  G and U1 are formed on threads 1..30 x
// 1..14, U2 on the inner 28 x 12 voxels.  Step j of each thread, walking a
// chunk of z planes:
//   A. forms G and U1 of plane j-1 (i/j neighbours of U0, D, B from shared
//      memory, k neighbours from its registers) and publishes U1;
//   B. forms U2 of plane j-2 from U1 (published in the previous step, k
//      neighbours in registers) and writes it;
//   C. publishes U0, Dx, Bx, Dy, By of plane j (loaded one step earlier).
// One barrier per plane; the i/j mirrors are neighbour offsets, the k mirrors
// selects.  The terms are summed in the reference's order.  HBM traffic: read
// U0, D, B, f; write U2 (36 B per voxel in 3D, 24 B in 2D) for two sweeps.
#include <type_traits>

#include "sb_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 4, OY = BY - 4;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

template <bool THREE, bool CHECK>
__global__ void __launch_bounds__(NT, 2) k_sb_sweep2(SbSweepArgs a, Dims d, int zc, const StopCtl* ctl,
                                                     double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU0[2][BY * BX];
    __shared__ float sU1[2][BY * BX];
    __shared__ float sDx[2][BY * BX];
    __shared__ float sBx[2][BY * BX];
    __shared__ float sDy[2][BY * BX];
    __shared__ float sBy[2][BY * BX];
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 2 && tx <= BX - 3 && ty >= 2 && ty <= BY - 3;
    // mirrored neighbours in the tile (SB_TV_core.c:262-269), clamped to it
    // where only unused halo values depend on them
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
    const int col = min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const float lam = a.lambda, mu = a.mu, norm = a.norm;
    float pa = 0.f, pb = 0.f;

    if constexpr (!THREE) {
        // SB_TV_core.c:166-170, twice
        const float u0 = __ldg(a.u + col), fv = __ldg(a.f + col);
        const float dx = __ldg(a.dd[0] + col), dy = __ldg(a.dd[1] + col);
        const float bx = __ldg(a.bb[0] + col), by = __ldg(a.bb[1] + col);
        sU0[0][oc] = u0;
        sDx[0][oc] = dx;
        sDy[0][oc] = dy;
        sBx[0][oc] = bx;
        sBy[0][oc] = by;
        __syncthreads();
        const float g = sDx[0][oxl] - dx + sDy[0][oyl] - dy - sBx[0][oxl] + bx - sBy[0][oyl] + by;
        float s = g;
        s += sU0[0][oxh] + sU0[0][oxl] + sU0[0][oyh] + sU0[0][oyl];
        s *= lam;
        s += mu * fv;
        const float u1 = norm * s;
        sU1[0][oc] = u1;
        __syncthreads();
        if (o_pt) {
            float s2 = g;
            s2 += sU1[0][oxh] + sU1[0][oxl] + sU1[0][oyh] + sU1[0][oyl];
            s2 *= lam;
            s2 += mu * fv;
            const float u2 = norm * s2;
            a.u2[col] = u2;
            if (CHECK) {
                const float df = u2 - u1;
                pa = df * df;
                pb = u2 * u2;
            }
        }
    } else {
        const int z0 = blockIdx.z * zc;
        const int z1 = min(z0 + zc, nz);
        const int sxy = (int)d.sxy;
        auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
        // inputs of plane j entering step j (c*), and of the planes below it
        const int o0 = at(z0), om1 = at(z0 - 1), om2 = at(z0 - 2);
        float cu0 = __ldg(a.u + o0), cf = __ldg(a.f + o0);
        float cdx = __ldg(a.dd[0] + o0), cdy = __ldg(a.dd[1] + o0), cdz = __ldg(a.dd[2] + o0);
        float cbx = __ldg(a.bb[0] + o0), cby = __ldg(a.bb[1] + o0), cbz = __ldg(a.bb[2] + o0);
        float pu0 = __ldg(a.u + om1), ppu0 = __ldg(a.u + om2);
        float pdz = __ldg(a.dd[2] + om1), pbz = __ldg(a.bb[2] + om1);
        float ppdz = __ldg(a.dd[2] + om2), ppbz = __ldg(a.bb[2] + om2);
        float pf = __ldg(a.f + om1), ppf = __ldg(a.f + om2);
        float pu1 = 0.f, ppu1 = 0.f, pg = 0.f;  // U1 of planes j-2, j-3; G of plane j-2
        // ring slot of plane p: (p - z0) & 1; plane z0-1 goes to slot 1
        sU0[1][oc] = pu0;
        sDx[1][oc] = __ldg(a.dd[0] + om1);
        sDy[1][oc] = __ldg(a.dd[1] + om1);
        sBx[1][oc] = __ldg(a.bb[0] + om1);
        sBy[1][oc] = __ldg(a.bb[1] + om1);
        __syncthreads();

        auto step = [&](auto par, auto full, int j) {
            constexpr int P = decltype(par)::value;
            constexpr bool FULL = decltype(full)::value;
            const int on = at(j + 1);  // prefetch plane j+1
            const float nu0 = __ldg(a.u + on), nf = __ldg(a.f + on);
            const float ndx = __ldg(a.dd[0] + on), ndy = __ldg(a.dd[1] + on), ndz = __ldg(a.dd[2] + on);
            const float nbx = __ldg(a.bb[0] + on), nby = __ldg(a.bb[1] + on), nbz = __ldg(a.bb[2] + on);
            // A. G and U1 of plane m = j-1 (SB_TV_core.c:273-280)
            const int m = j - 1;
            const float dzl = (m == 0) ? cdz : ppdz;  // mirrored k-1
            const float bzl = (m == 0) ? cbz : ppbz;
            const float dval = sDx[1 - P][oxl] - sDx[1 - P][oc] + sDy[1 - P][oyl] - sDy[1 - P][oc] + dzl - pdz;
            const float bval = -sBx[1 - P][oxl] + sBx[1 - P][oc] - sBy[1 - P][oyl] + sBy[1 - P][oc] - bzl + pbz;
            const float g = dval + bval;
            const float zh0 = (m == nz - 1) ? ppu0 : cu0, zl0 = (m == 0) ? cu0 : ppu0;
            float s = g;
            s += sU0[1 - P][oxh] + sU0[1 - P][oxl] + sU0[1 - P][oyh] + sU0[1 - P][oyl] + zh0 + zl0;
            s *= lam;
            s += mu * pf;
            const float u1 = norm * s;
            sU1[1 - P][oc] = u1;
            // B. U2 of plane kf = j-2
            if (FULL) {
                const int kf = j - 2;
                const float zh1 = (kf == nz - 1) ? ppu1 : u1, zl1 = (kf == 0) ? u1 : ppu1;
                float s2 = pg;
                s2 += sU1[P][oxh] + sU1[P][oxl] + sU1[P][oyh] + sU1[P][oyl] + zh1 + zl1;
                s2 *= lam;
                s2 += mu * ppf;
                const float u2 = norm * s2;
                if (o_pt) a.u2[kf * sxy + col] = u2;
                if (CHECK && o_pt) {
                    const float df = u2 - pu1;
                    pa += df * df;
                    pb += u2 * u2;
                }
            }
            // C. publish plane j
            sU0[P][oc] = cu0;
            sDx[P][oc] = cdx;
            sDy[P][oc] = cdy;
            sBx[P][oc] = cbx;
            sBy[P][oc] = cby;
            __syncthreads();
            ppu0 = pu0;
            pu0 = cu0;
            cu0 = nu0;
            ppdz = pdz;
            pdz = cdz;
            cdz = ndz;
            ppbz = pbz;
            pbz = cbz;
            cbz = nbz;
            cdx = ndx;
            cdy = ndy;
            cbx = nbx;
            cby = nby;
            ppf = pf;
            pf = cf;
            cf = nf;
            ppu1 = pu1;
            pu1 = u1;
            pg = g;
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

// shrinkage of v = grad U + B_prev into D, and the Bregman update B = v - D
// (SB_TV_core.c:284-371): anisotropic per component, isotropic on |v|
template <bool THREE, bool ANISO>
__device__ __forceinline__ void sb_shrink(float g1, float g2, float g3, float b1, float b2, float b3, float dlam,
                                          float& d1, float& d2, float& d3, float& n1, float& n2, float& n3) {
    const float v1 = g1 + b1, v2 = g2 + b2, v3 = THREE ? g3 + b3 : 0.f;
    if (ANISO) {
        // (v / |v|) * max(|v| - 1/lambda, 0), 0 for v == 0: the same value as a sign copy
        d1 = copysignf(fmaxf(fabsf(v1) - dlam, 0.f), v1);
        d2 = copysignf(fmaxf(fabsf(v2) - dlam, 0.f), v2);
        d3 = THREE ? copysignf(fmaxf(fabsf(v3) - dlam, 0.f), v3) : 0.f;
    } else {
        const float den = THREE ? sqrtf(v1 * v1 + v2 * v2 + v3 * v3) : sqrtf(v1 * v1 + v2 * v2);
        const float m = fmaxf(den - dlam, 0.f);
        const float r = (den != 0.f) ? __frcp_rn(den) : 0.f;  // v / den as v * (1/den), within 1 ulp
        d1 = m * (v1 * r);
        d2 = m * (v2 * r);
        d3 = m * (v3 * r);
    }
    // B += (grad U) - D, summed as the reference does (SB_TV_core.c:366-368)
    n1 = b1 + (g1 - d1);
    n2 = b2 + (g2 - d2);
    n3 = THREE ? b3 + (g3 - d3) : 0.f;
}

// One whole split-Bregman outer iteration k >= 1 in one streaming pass.  The
// split variable is a function of the state: D^k = shrink(grad U^k + B^{k-1}),
// B^k = B^{k-1} + grad U^k - D^k, so D is never stored; the pass reads U^k,
// B^{k-1} and f, forms D^k and B^k on the fly, runs both Jacobi sweeps with
// them and writes U^{k+1} and B^k (36 B per voxel in 3D, against 78 B for the
// sweep pass plus a separate shrinkage pass).  Step j, with the tile and
// halo of k_sb_sweep2 (D and B are needed one voxel further out, at i-1 and
// j-1 of the sweep's halo, and need U one voxel beyond them at i+1, j+1):
//   A0. forms D^k, B^k of plane j-1 (i/j successors of U^k from shared memory,
//       k successor from registers); publishes Dx, Dy, Bx, By; writes B^k;
//   A.  forms G and U1 of plane j-2 and publishes U1;
//   B.  forms U2 of plane j-3 and writes it;
//   C.  publishes U^k of plane j (loaded one step earlier).
template <bool THREE, bool CHECK, bool ANISO>
__global__ void __launch_bounds__(NT, 2) k_sb_fused(SbFusedArgs a, Dims d, int zc, const StopCtl* ctl,
                                                    double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU0[4][BY * BX];
    __shared__ float sU1[2][BY * BX];
    __shared__ float sDx[2][BY * BX];
    __shared__ float sBx[2][BY * BX];
    __shared__ float sDy[2][BY * BX];
    __shared__ float sBy[2][BY * BX];
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 2 && tx <= BX - 3 && ty >= 2 && ty <= BY - 3;
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
    const int col = min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const float lam = a.lambda, mu = a.mu, norm = a.norm, dlam = a.dlam;
    float pa = 0.f, pb = 0.f;

    if constexpr (!THREE) {
        // one plane: D, B from U and B_prev; both sweeps (SB_TV_core.c:166-248);
        // every load issued before the first barrier
        const float u0 = __ldg(a.u + col), fv = __ldg(a.f + col);
        const float bp1 = __ldg(a.bp[0] + col), bp2 = __ldg(a.bp[1] + col);
        sU0[0][oc] = u0;
        __syncthreads();
        float dx, dy, dz, bx, by, bz;
        sb_shrink<false, ANISO>(sU0[0][oxh] - u0, sU0[0][oyh] - u0, 0.f, bp1, bp2, 0.f, dlam, dx, dy, dz, bx, by,
                                bz);
        if (o_pt) {
            a.bn[0][col] = bx;
            a.bn[1][col] = by;
        }
        sDx[0][oc] = dx;
        sDy[0][oc] = dy;
        sBx[0][oc] = bx;
        sBy[0][oc] = by;
        __syncthreads();
        const float g = sDx[0][oxl] - dx + sDy[0][oyl] - dy - sBx[0][oxl] + bx - sBy[0][oyl] + by;
        float s = g;
        s += sU0[0][oxh] + sU0[0][oxl] + sU0[0][oyh] + sU0[0][oyl];
        s *= lam;
        s += mu * fv;
        const float u1 = norm * s;
        sU1[0][oc] = u1;
        __syncthreads();
        if (o_pt) {
            float s2 = g;
            s2 += sU1[0][oxh] + sU1[0][oxl] + sU1[0][oyh] + sU1[0][oyl];
            s2 *= lam;
            s2 += mu * fv;
            const float u2 = norm * s2;
            a.u2[col] = u2;
            if (CHECK) {
                const float df = u2 - u1;
                pa = df * df;
                pb = u2 * u2;
            }
        }
    } else {
        const int z0 = blockIdx.z * zc;
        const int z1 = min(z0 + zc, nz);
        const int sxy = (int)d.sxy;
        auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
        // registers entering step j: U^k of planes j, j-1, j-2, j-3; B^{k-1} of
        // plane j-1; Dz, Bz of planes j-2, j-3; G of plane j-3; U1 of planes
        // j-3, j-4
        float cu = __ldg(a.u + at(z0 - 1)), pu = __ldg(a.u + at(z0 - 2)), ppu = __ldg(a.u + at(z0 - 3));
        float pppu = 0.f;
        float cb1 = __ldg(a.bp[0] + at(z0 - 2)), cb2 = __ldg(a.bp[1] + at(z0 - 2)), cb3 = __ldg(a.bp[2] + at(z0 - 2));
        float dzb = 0.f, bzb = 0.f, dzc = 0.f, bzc = 0.f;
        float gc = 0.f, u1c = 0.f, u1d = 0.f;
        // f of planes j-1, j-2, j-3 entering step j = z0 - 1
        float fa = __ldg(a.f + at(z0 - 2)), fb = __ldg(a.f + at(z0 - 3)), fc = 0.f;
        // U ring slot of plane p: (p - z0 + 4) & 3; D/B and U1 slots: (p - z0 + 4) & 1
        sU0[2][oc] = pu;  // plane z0-2
        __syncthreads();

        // R = (j - z0 + 1) & 3 for step j (steps start at j = z0 - 1)
        auto step = [&](auto rr, auto full, int j) {
            constexpr int R = decltype(rr)::value;
            constexpr bool FULL = decltype(full)::value;
            constexpr int SJ = (R + 3) & 3, SM1 = (R + 2) & 3, SM2 = (R + 1) & 3;  // U slots of j, j-1, j-2
            constexpr int W1 = (R + 2) & 1, W2 = (R + 1) & 1, W3 = R & 1;         // parity slots of j-1, j-2, j-3
            const int on = at(j + 1);
            const float nu = __ldg(a.u + on);
            const int ob = at(j);
            const float nb1 = __ldg(a.bp[0] + ob), nb2 = __ldg(a.bp[1] + ob), nb3 = __ldg(a.bp[2] + ob);
            const float nf = __ldg(a.f + ob);
            // A0. D^k, B^k of plane m0 = j-1
            float dx, dy, dza, bx, by, bza;
            {
                const int m0 = j - 1;
                const float zhi = (m0 == nz - 1) ? ppu : cu;  // mirrored k+1 (SB_TV_core.c:293)
                const float* U1s = sU0[SM1];
                sb_shrink<true, ANISO>(U1s[oxh] - pu, U1s[oyh] - pu, zhi - pu, cb1, cb2, cb3, dlam, dx, dy, dza, bx,
                                       by, bza);
                if (o_pt && m0 >= z0 && m0 < z1) {
                    const int v = m0 * sxy + col;
                    a.bn[0][v] = bx;
                    a.bn[1][v] = by;
                    a.bn[2][v] = bza;
                }
                sDx[W1][oc] = dx;
                sDy[W1][oc] = dy;
                sBx[W1][oc] = bx;
                sBy[W1][oc] = by;
            }
            // A. G and U1 of plane m = j-2 (SB_TV_core.c:273-280); its D, B were
            // published in the previous step
            const int m = j - 2;
            const float dzl = (m == 0) ? dza : dzc;  // mirrored k-1
            const float bzl = (m == 0) ? bza : bzc;
            const float dval = sDx[W2][oxl] - sDx[W2][oc] + sDy[W2][oyl] - sDy[W2][oc] + dzl - dzb;
            const float bval = -sBx[W2][oxl] + sBx[W2][oc] - sBy[W2][oyl] + sBy[W2][oc] - bzl + bzb;
            const float g = dval + bval;
            const float* Um = sU0[SM2];
            const float zh0 = (m == nz - 1) ? pppu : pu, zl0 = (m == 0) ? pu : pppu;
            float s = g;
            s += Um[oxh] + Um[oxl] + Um[oyh] + Um[oyl] + zh0 + zl0;
            s *= lam;
            s += mu * fb;
            const float u1 = norm * s;
            sU1[W2][oc] = u1;
            // B. U2 of plane kf = j-3
            if (FULL) {
                const int kf = j - 3;
                const float zh1 = (kf == nz - 1) ? u1d : u1, zl1 = (kf == 0) ? u1 : u1d;
                float s2 = gc;
                s2 += sU1[W3][oxh] + sU1[W3][oxl] + sU1[W3][oyh] + sU1[W3][oyl] + zh1 + zl1;
                s2 *= lam;
                s2 += mu * fc;
                const float u2 = norm * s2;
                if (o_pt) a.u2[kf * sxy + col] = u2;
                if (CHECK && o_pt) {
                    const float df = u2 - u1c;
                    pa += df * df;
                    pb += u2 * u2;
                }
            }
            // C. publish U^k of plane j
            sU0[SJ][oc] = cu;
            __syncthreads();
            pppu = ppu;
            ppu = pu;
            pu = cu;
            cu = nu;
            cb1 = nb1;
            cb2 = nb2;
            cb3 = nb3;
            dzc = dzb;
            bzc = bzb;
            dzb = dza;
            bzb = bza;
            gc = g;
            u1d = u1c;
            u1c = u1;
            fc = fb;
            fb = fa;
            fa = nf;
        };
        step(Ic<0>{}, std::false_type{}, z0 - 1);
        step(Ic<1>{}, std::false_type{}, z0);
        step(Ic<2>{}, std::false_type{}, z0 + 1);
        step(Ic<3>{}, std::false_type{}, z0 + 2);
        int j = z0 + 3;
        for (; j + 3 <= z1 + 2; j += 4) {
            step(Ic<0>{}, std::true_type{}, j);
            step(Ic<1>{}, std::true_type{}, j + 1);
            step(Ic<2>{}, std::true_type{}, j + 2);
            step(Ic<3>{}, std::true_type{}, j + 3);
        }
        if (j <= z1 + 2) step(Ic<0>{}, std::true_type{}, j);
        if (j + 1 <= z1 + 2) step(Ic<1>{}, std::true_type{}, j + 1);
        if (j + 2 <= z1 + 2) step(Ic<2>{}, std::true_type{}, j + 2);
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

}  // namespace

SbPlan sb_sweep2_plan(const Dims& d) {
    SbPlan T;
    const char* e = getenv("CILREG_SB_KERNEL");
    // "simple" selects the per-sweep kernels; volumes of 2^31 voxels or more
    // use them too (this kernel indexes with 32-bit offsets)
    T.use = !(e && e[0] == 's') && d.n < (1LL << 31);
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_sb_sweep2<true, false>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int sb_sweep2_step(const SbPlan& T, const SbSweepArgs& a, const Dims& d, const StopCtl* ctl, int check,
                   double2* partials, cudaStream_t s) {
    const bool three = d.nz > 1;
    auto kern = three ? (check ? k_sb_sweep2<true, true> : k_sb_sweep2<true, false>)
                      : (check ? k_sb_sweep2<false, true> : k_sb_sweep2<false, false>);
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg

namespace cilreg {

int sb_fused_step(const SbPlan& T, const SbFusedArgs& a, bool aniso, const Dims& d, const StopCtl* ctl, int check,
                  double2* partials, cudaStream_t s) {
    const bool three = d.nz > 1;
    decltype(&k_sb_fused<true, true, true>) kern;
    if (three)
        kern = check ? (aniso ? k_sb_fused<true, true, true> : k_sb_fused<true, true, false>)
                     : (aniso ? k_sb_fused<true, false, true> : k_sb_fused<true, false, false>);
    else
        kern = check ? (aniso ? k_sb_fused<false, true, true> : k_sb_fused<false, true, false>)
                     : (aniso ? k_sb_fused<false, false, true> : k_sb_fused<false, false, false>);
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
