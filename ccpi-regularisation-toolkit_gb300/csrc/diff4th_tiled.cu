// Fourth-order diffusion iteration as a 2.5D streaming stencil (2D images are
// the nz == 1 case).  Reference arithmetic: Diffus4th_order_core.c:103-265.
//
// The update needs the weighted Laplacian W at the voxel and its mirrored
// neighbours; W needs U on the mirrored 19-point neighbourhood.  A CTA of
// 32 x 24 threads holds an overlapping tile (thread (tx, ty) on voxel
// (x0 - 2 + tx, y0 - 2 + ty)); W is formed on the inner 30 x 22 voxels, the
// update on the inner 28 x 20.  Step j of each thread:
//   B. publishes U(j) into a four-plane shared-memory ring;
//   A. after the barrier, forms W(j-1) once per voxel from planes j-2, j-1, j
//      of the ring (mirrored in all three axes) into shared memory;
//   C. updates plane j-2 from W of planes j-3, j-2, j-1 (z from registers,
//      x/y from shared memory).
// One barrier per plane.  HBM traffic: read U and f, write U (12 B/voxel);
// the reference's two sweeps move 24 B and store W.  The kernel is bound by
// instruction issue and latency: at 40 registers two 768-thread CTAs (48
// warps) fit on an SM.  The 24-row tile spends 1.37 thread-steps per updated
// voxel against 1.52 for 16 rows (1.30 -> 1.26 ms per 512^3 iteration).
#include <stdlib.h>

#include <type_traits>

#include "diff4th_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 24;
constexpr int OX = BX - 4, OY = BY - 4;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

// CHECK: a stopping-check iteration (per-CTA partial sums).  IT: element-offset
// type (int below 2^31 voxels).
template <bool THREE, bool CHECK, typename IT>
__global__ void __launch_bounds__(NT, 2) k_d4_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                     const float* __restrict__ F, float lam, float tau, float isg2,
                                                     Dims d, int zc, const StopCtl* ctl, double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU[4][BY][BX];
    __shared__ float sW[2][BY][BX];
    if (ctl->stop) return;
    const float EPS = 1.0e-7f;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool w_pt = in_xy && tx >= 1 && tx <= BX - 2 && ty >= 1 && ty <= BY - 2;
    const bool o_pt = in_xy && tx >= 2 && tx <= BX - 3 && ty >= 2 && ty <= BY - 3;
    const int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    const int xl = (nx == 1) ? tx : ((x - 1 < 0) ? tx + 1 : tx - 1);
    const int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    const int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    const IT col = in_xy ? ((IT)y * nx + x) : 0;
    const IT sxy = (IT)d.sxy;
    auto ld = [&](const float* p, int k) -> float {
        return (in_xy && k >= 0 && k < nz) ? __ldg(p + ((IT)k * sxy + col)) : 0.f;
    };

    float wa = 0.f, wb = 0.f, wc = 0.f;  // W of planes j-1, j-2, j-3 at this voxel
    float pa = 0.f, pb = 0.f;
    // U ring slot of plane p: (p - z0 + 4) & 3; W ring slot: (p - z0 + 2) & 1
    sU[2][ty][tx] = ld(U, z0 - 2);
    sU[3][ty][tx] = ld(U, z0 - 1);
    float uj = ld(U, z0);
    float fa = o_pt ? ld(F, z0 - 2) : 0.f, fb = o_pt ? ld(F, z0 - 1) : 0.f;  // f of planes j-2, j-1

    // R = (j - z0) & 3
    auto step = [&](auto rr, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // W slots of planes j-1, j-2
        const float un1 = (j + 1 <= z1 + 1) ? ld(U, j + 1) : 0.f;  // prefetch U(j+1)
        const float fn = o_pt ? ld(F, j) : 0.f;                      // prefetch f(j)
        // B. publish U(j)
        sU[SJ][ty][tx] = uj;
        __syncthreads();
        // A. weighted Laplacian of plane m = j-1 (Diffus4th_order_core.c:176-235)
        const int m = j - 1;
        wc = wb;
        wb = wa;
        wa = 0.f;
        if (m >= 0 && m < nz && m >= z0 - 1 && m <= z1 && w_pt) {
            const float c0 = sU[SM][ty][tx];
            const float um_x = sU[SM][ty][xl], up_x = sU[SM][ty][xh];
            const float um_y = sU[SM][yl][tx], up_y = sU[SM][yh][tx];
            const float gx = 0.5f * (um_x - up_x), gy = 0.5f * (um_y - up_y);
            const float gx2 = gx * gx, gy2 = gy * gy;
            const float gxx = um_x + up_x - 2.0f * c0;
            const float gyy = um_y + up_y - 2.0f * c0;
            const float gxy = 0.25f * (sU[SM][yl][xl] + sU[SM][yh][xh] - sU[SM][yh][xl] - sU[SM][yl][xh]);
            const float xy2 = 2.0f * gx * gy * gxy;
            float den, vn, vo;
            if (THREE) {
                // mirrored k-1 / k+1 planes (an axis of length 1 maps to itself)
                const float(*pl)[BX] = (nz == 1) ? sU[SM] : ((m == 0) ? sU[SJ] : sU[SM2]);
                const float(*ph)[BX] = (nz == 1) ? sU[SM] : ((m == nz - 1) ? sU[SM2] : sU[SJ]);
                const float zm = pl[ty][tx], zp = ph[ty][tx];
                const float gz = 0.5f * (zm - zp);
                const float gz2 = gz * gz;
                const float gzz = zm + zp - 2.0f * c0;
                const float gxz = 0.25f * (pl[ty][xl] - pl[ty][xh] - ph[ty][xl] + ph[ty][xh]);
                const float gyz = 0.25f * (pl[yl][tx] - pl[yh][tx] - ph[yl][tx] + ph[yh][tx]);
                const float xz2 = 2.0f * gx * gz * gxz;
                const float yz2 = 2.0f * gy * gz * gyz;
                den = gx2 + gy2 + gz2;
                const float nn = gxx * gx2 + gyy * gy2 + gzz * gz2 + xy2 + xz2 + yz2;
                const float oo = (gy2 + gz2) * gxx + (gx2 + gz2) * gyy + (gx2 + gy2) * gzz - xy2 - xz2 - yz2;
                const float iq = __frcp_rn((den <= EPS) ? EPS : den);
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
            wa = (c * c) * vn + c * vo;
            sW[WM][ty][tx] = wa;
        }
        // C. update plane kf = j-2 (Diffus4th_order_core.c:237-265); its W was
        // published in the previous step
        const int kf = j - 2;
        if (o_pt && kf >= z0 && kf < z1) {
            const float w = sW[WK][ty][tx];
            const float lx = sW[WK][ty][xl] + sW[WK][ty][xh] - 2.0f * w;
            const float ly = sW[WK][yl][tx] + sW[WK][yh][tx] - 2.0f * w;
            float lap = lx + ly;
            if (THREE) {
                const float wlo = (nz == 1) ? w : ((kf == 0) ? wa : wc);        // mirrored W(k-1)
                const float whi = (nz == 1) ? w : ((kf == nz - 1) ? wc : wa);   // mirrored W(k+1)
                lap = lap + (wlo + whi - 2.0f * w);
            }
            const float u = sU[SM2][ty][tx];
            const float un = u + tau * (-lam * lap - (u - fa));
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
    int j = z0;
    for (; j + 3 <= z1 + 1; j += 4) {
        step(Ic<0>{}, j);
        step(Ic<1>{}, j + 1);
        step(Ic<2>{}, j + 2);
        step(Ic<3>{}, j + 3);
    }
    if (j <= z1 + 1) step(Ic<0>{}, j);
    if (j + 1 <= z1 + 1) step(Ic<1>{}, j + 1);
    if (j + 2 <= z1 + 1) step(Ic<2>{}, j + 2);
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// ---------------------------------------------------------------------------
// 3D column kernel: fewer instructions per voxel.
//
// A CTA of 32 x 8 threads covers a 32 x 32 tile (updated: the inner 28 x 28).
// Thread (tx, ty) owns the column of four rows 4 ty .. 4 ty + 3 at x =
// x0 - 2 + tx, and keeps the U, W and f of its own rows in registers across
// planes.  Vertical neighbours of its rows are its own registers except the
// rows just above and below its column (two shared-memory reads per plane
// and array); horizontal neighbours come from the adjacent lanes of the warp
// (a warp is one tile row of 32 voxels) by shuffles.  Per plane j: load and
// publish U(j) of the four rows, one barrier, W(j-1) of the four rows
// (published for the neighbours' update), then the update of plane j-2.
// W and the update use the same expressions, in the same order, as
// k_d4_stream; only where the neighbour values come from differs.
constexpr int CX = 32, CTY = 32;  // tile: 32 x 32 voxels
constexpr int CQX = CX - 4, CQY = CTY - 4;

// RR rows per thread (CTY / RR thread rows), MINB CTAs per SM
template <int RR, int MINB, bool CHECK>
__global__ void __launch_bounds__(CX * (CTY / RR), MINB)
    k_d4_cols(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam, float tau,
              float isg2, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    constexpr int CNT = CX * (CTY / RR);
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ float sU[4][CTY][CX];
    __shared__ float sW[2][CTY][CX];
    if (ctl->stop) return;
    const float EPS = 1.0e-7f;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * CQX + tx - 2;
    const int ybase = blockIdx.y * CQY + RR * ty - 2;  // y of row 0 of this thread
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const int sxy = d.sxy;
    const bool in_x = (x >= 0) && (x < nx);
    const bool wx = in_x && tx >= 1 && tx <= CX - 2;
    const bool ox = in_x && tx >= 2 && tx <= CX - 3;
    // horizontal mirror: which lane holds the lower / upper neighbour
    const bool x_self = (nx == 1);
    const bool xlo_m = (x - 1 < 0), xhi_m = (x + 1 >= nx);
    const int xc = min(max(x, 0), nx - 1);
    // rows of the column: offsets (clamped into the volume: halo rows outside
    // it load the nearest voxel, never used unmirrored) and mirror flags
    int roff[RR];
    bool wrow[RR], orow[RR], ylo_m[RR], yhi_m[RR];
#pragma unroll
    for (int r = 0; r < RR; r++) {
        const int y = ybase + r, tr = RR * ty + r;
        roff[r] = min(max(y, 0), ny - 1) * nx + xc;
        const bool in_y = (y >= 0) && (y < ny);
        wrow[r] = wx && in_y && tr >= 1 && tr <= CTY - 2;
        orow[r] = ox && in_y && tr >= 2 && tr <= CTY - 3;
        ylo_m[r] = (ny == 1) ? false : (y - 1 < 0);
        yhi_m[r] = (ny == 1) ? false : (y + 1 >= ny);
    }
    const bool y_self = (ny == 1);
    const int rup = max(RR * ty - 1, 0), rdn = min(RR * ty + RR, CTY - 1);  // tile rows just above / below
    auto ldu = [&](int k, int r) -> float { return __ldg(U + ((long long)min(max(k, 0), nz - 1) * sxy + roff[r])); };
    auto ldf = [&](int k, int r) -> float { return __ldg(F + ((long long)min(max(k, 0), nz - 1) * sxy + roff[r])); };
    // the horizontal neighbours of v (mirrored at the volume edge)
    auto xnb = [&](float v, float& lo, float& hi) {
        const float a = __shfl_up_sync(0xffffffffu, v, 1);    // lane tx - 1
        const float b = __shfl_down_sync(0xffffffffu, v, 1);  // lane tx + 1
        lo = x_self ? v : (xlo_m ? b : a);
        hi = x_self ? v : (xhi_m ? a : b);
    };

    float u2[RR], u1[RR], u0[RR], un[RR];  // U of planes j-2, j-1, j (own rows) and the prefetch of j+1
    float wa[RR], wb[RR], wc[RR];          // W of planes j-1, j-2, j-3
    float pa = 0.f, pb = 0.f;
#pragma unroll
    for (int r = 0; r < RR; r++) {
        u2[r] = ldu(z0 - 2, r);
        u1[r] = ldu(z0 - 1, r);
        u0[r] = ldu(z0, r);
        wa[r] = wb[r] = wc[r] = 0.f;
        sU[2][RR * ty + r][tx] = u2[r];
        sU[3][RR * ty + r][tx] = u1[r];
    }

    auto step = [&](auto rr, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // W slots of planes j-1, j-2
        float fa[RR];  // f of plane j-2, used by the update after the barrier and W
#pragma unroll
        for (int r = 0; r < RR; r++) {
            un[r] = ldu(j + 1, r);  // prefetch U(j+1)
            fa[r] = orow[r] ? ldf(j - 2, r) : 0.f;
            sU[SJ][RR * ty + r][tx] = u0[r];  // B. publish U(j)
        }
        __syncthreads();
        // A. W of plane m = j-1 for the four rows (Diffus4th_order_core.c:176-235)
        const int m = j - 1;
        const bool m_ok = (m >= 0) && (m < nz) && (m >= z0 - 1) && (m <= z1);
        // planes m-1 (pl) and m+1 (ph), mirrored at the first and last plane
        const bool pl_is_j = (m == 0), ph_is_j2 = (m == nz - 1);
        float c[RR + 2], pl[RR + 2], ph[RR + 2];  // rows -1 .. RR of the column (index + 1)
        c[0] = sU[SM][rup][tx];
        c[RR + 1] = sU[SM][rdn][tx];
        pl[0] = pl_is_j ? sU[SJ][rup][tx] : sU[SM2][rup][tx];
        pl[RR + 1] = pl_is_j ? sU[SJ][rdn][tx] : sU[SM2][rdn][tx];
        ph[0] = ph_is_j2 ? sU[SM2][rup][tx] : sU[SJ][rup][tx];
        ph[RR + 1] = ph_is_j2 ? sU[SM2][rdn][tx] : sU[SJ][rdn][tx];
#pragma unroll
        for (int r = 0; r < RR; r++) {
            c[r + 1] = u1[r];
            pl[r + 1] = pl_is_j ? u0[r] : u2[r];
            ph[r + 1] = ph_is_j2 ? u2[r] : u0[r];
        }
        float cl[RR + 2], ch[RR + 2];  // horizontal neighbours of every row of plane m
#pragma unroll
        for (int q = 0; q < RR + 2; q++) xnb(c[q], cl[q], ch[q]);
#pragma unroll
        for (int r = 0; r < RR; r++) {
            float pll, plh, phl, phh;  // horizontal neighbours of pl, ph on this row
            xnb(pl[r + 1], pll, plh);
            xnb(ph[r + 1], phl, phh);
            // the mirrored rows above / below of array v at row r (selects
            // between constant indices: the arrays stay in registers)
            auto lo = [&](const float* v) { return y_self ? v[r + 1] : (ylo_m[r] ? v[r + 2] : v[r]); };
            auto hi = [&](const float* v) { return y_self ? v[r + 1] : (yhi_m[r] ? v[r] : v[r + 2]); };
            wc[r] = wb[r];
            wb[r] = wa[r];
            wa[r] = 0.f;
            if (m_ok && wrow[r]) {
                const float c0 = c[r + 1];
                const float um_x = cl[r + 1], up_x = ch[r + 1];
                const float um_y = lo(c), up_y = hi(c);
                const float gx = 0.5f * (um_x - up_x), gy = 0.5f * (um_y - up_y);
                const float gx2 = gx * gx, gy2 = gy * gy;
                const float gxx = um_x + up_x - 2.0f * c0;
                const float gyy = um_y + up_y - 2.0f * c0;
                const float gxy = 0.25f * (lo(cl) + hi(ch) - hi(cl) - lo(ch));
                const float xy2 = 2.0f * gx * gy * gxy;
                const float zm = pl[r + 1], zp = ph[r + 1];
                const float gz = 0.5f * (zm - zp);
                const float gz2 = gz * gz;
                const float gzz = zm + zp - 2.0f * c0;
                const float gxz = 0.25f * (pll - plh - phl + phh);
                const float gyz = 0.25f * (lo(pl) - hi(pl) - lo(ph) + hi(ph));
                const float xz2 = 2.0f * gx * gz * gxz;
                const float yz2 = 2.0f * gy * gz * gyz;
                const float den = gx2 + gy2 + gz2;
                const float nn = gxx * gx2 + gyy * gy2 + gzz * gz2 + xy2 + xz2 + yz2;
                const float oo = (gy2 + gz2) * gxx + (gx2 + gz2) * gyy + (gx2 + gy2) * gzz - xy2 - xz2 - yz2;
                const float iq = __frcp_rn((den <= EPS) ? EPS : den);
                const float vn = nn * iq, vo = oo * iq;
                const float cc = __frcp_rn(1.0f + den * isg2);
                wa[r] = (cc * cc) * vn + cc * vo;
            }
            sW[WM][RR * ty + r][tx] = wa[r];
        }
        // C. update plane kf = j-2 (Diffus4th_order_core.c:237-265); W of
        // plane j-2 of the rows above and below was published last step
        const int kf = j - 2;
        if (kf >= z0 && kf < z1) {
            float w[RR + 2];
            w[0] = sW[WK][rup][tx];
            w[RR + 1] = sW[WK][rdn][tx];
#pragma unroll
            for (int r = 0; r < RR; r++) w[r + 1] = wb[r];
#pragma unroll
            for (int r = 0; r < RR; r++) {
                float wl, wh;
                xnb(wb[r], wl, wh);
                const float wlo_y = y_self ? w[r + 1] : (ylo_m[r] ? w[r + 2] : w[r]);
                const float whi_y = y_self ? w[r + 1] : (yhi_m[r] ? w[r] : w[r + 2]);
                if (orow[r]) {
                    const float wv = w[r + 1];
                    const float lx = wl + wh - 2.0f * wv;
                    const float ly = wlo_y + whi_y - 2.0f * wv;
                    float lap = lx + ly;
                    const float wlo = (nz == 1) ? wv : ((kf == 0) ? wa[r] : wc[r]);       // mirrored W(k-1)
                    const float whi = (nz == 1) ? wv : ((kf == nz - 1) ? wc[r] : wa[r]);  // mirrored W(k+1)
                    lap = lap + (wlo + whi - 2.0f * wv);
                    const float u = u2[r];
                    const float unv = u + tau * (-lam * lap - (u - fa[r]));
                    Un[(long long)kf * sxy + roff[r]] = unv;
                    if (CHECK) {
                        const float df = unv - u;
                        pa += df * df;
                        pb += unv * unv;
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < RR; r++) {
            u2[r] = u1[r];
            u1[r] = u0[r];
            u0[r] = un[r];
        }
    };
    int j = z0;
    for (; j + 3 <= z1 + 1; j += 4) {
        step(Ic<0>{}, j);
        step(Ic<1>{}, j + 1);
        step(Ic<2>{}, j + 2);
        step(Ic<3>{}, j + 3);
    }
    if (j <= z1 + 1) step(Ic<0>{}, j);
    if (j + 1 <= z1 + 1) step(Ic<1>{}, j + 1);
    if (j + 2 <= z1 + 1) step(Ic<2>{}, j + 2);
    if (CHECK) block_pair_partial<CNT>(pa, pb, partials, block_slot());
}

bool use_d4_cols(const Dims& d) {
    const char* e = getenv("CILREG_D4_KERNEL");  // "rows": the one-voxel-per-thread kernel
    return d.nz > 1 && d.n < (1LL << 31) && !(e && e[0] == 'r');
}

// the column kernel's shape: CILREG_D4_COLS = 2 (two rows per thread, 512
// threads) or 4 (four rows, 256 threads; default)
constexpr int D4_RR = 4, D4_MINB = 2;
int d4_cols_rows() {
    const char* e = getenv("CILREG_D4_COLS");
    return (e && e[0] == '2') ? 2 : D4_RR;
}

}  // namespace

D4Plan d4_stream_plan(const Dims& d) {
    D4Plan T;
    if (use_d4_cols(d)) {
        T.cols = d4_cols_rows();
        T.block = dim3(CX, CTY / T.cols, 1);
        const int resident = (T.cols == 2) ? resident_ctas(k_d4_cols<2, 2, false>, CX * CTY / 2)
                                           : resident_ctas(k_d4_cols<D4_RR, D4_MINB, false>, CX * CTY / D4_RR);
        const long long tiles = (long long)((d.nx + CQX - 1) / CQX) * ((d.ny + CQY - 1) / CQY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
        T.grid = dim3((d.nx + CQX - 1) / CQX, (d.ny + CQY - 1) / CQY, (d.nz + T.zchunk - 1) / T.zchunk);
        T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
        return T;
    }
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_d4_stream<true, false, int>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int d4_stream_step(const D4Plan& T, const float* cur, float* nxt, const float* f, float lam, float tau, float isg2,
                   const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    const bool three = d.nz > 1;
    if (T.cols) {
        auto kc = (T.cols == 2) ? (check ? k_d4_cols<2, 2, true> : k_d4_cols<2, 2, false>)
                                : (check ? k_d4_cols<D4_RR, D4_MINB, true> : k_d4_cols<D4_RR, D4_MINB, false>);
        CILREG_CUDA(launch_pdl(kc, T.grid, T.block, 0, s, cur, nxt, f, lam, tau, isg2, d, T.zchunk, ctl, partials));
        return OK;
    }
    decltype(&k_d4_stream<true, true, int>) kern;
    if (d.n < (1LL << 31))
        kern = three ? (check ? k_d4_stream<true, true, int> : k_d4_stream<true, false, int>)
                     : (check ? k_d4_stream<false, true, int> : k_d4_stream<false, false, int>);
    else
        kern = three ? (check ? k_d4_stream<true, true, long long> : k_d4_stream<true, false, long long>)
                     : (check ? k_d4_stream<false, true, long long> : k_d4_stream<false, false, long long>);
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, cur, nxt, f, lam, tau, isg2, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
