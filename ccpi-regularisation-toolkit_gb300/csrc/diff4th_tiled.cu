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

    // the steps whose planes are all inside the volume and the chunk, none of
    // them the first or last plane of the volume: no plane check, no
    // mirrored-plane select and no load predicate (halo threads outside the
    // volume load voxel 0 of the plane, and never use it)
    const int js0 = max(z0 + 2, 3), js1 = min(z1, nz - 2);  // steady steps: js0 <= j <= js1 (3D)
    // R = (j - z0) & 3; ST: a steady step
    auto step = [&](auto rr, auto st, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr bool ST = THREE && decltype(st)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // W slots of planes j-1, j-2
        float un1, fn;
        if (ST) {
            un1 = __ldg(U + ((IT)(j + 1) * sxy + col));  // prefetch U(j+1)
            fn = __ldg(F + ((IT)j * sxy + col));         // prefetch f(j)
        } else {
            un1 = (j + 1 <= z1 + 1) ? ld(U, j + 1) : 0.f;
            fn = o_pt ? ld(F, j) : 0.f;
        }
        // B. publish U(j)
        sU[SJ][ty][tx] = uj;
        __syncthreads();
        // A. weighted Laplacian of plane m = j-1 (Diffus4th_order_core.c:176-235)
        const int m = j - 1;
        wc = wb;
        wb = wa;
        wa = 0.f;
        if ((ST || (m >= 0 && m < nz && m >= z0 - 1 && m <= z1)) && w_pt) {
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
                const float(*pl)[BX] = ST ? sU[SM2] : ((nz == 1) ? sU[SM] : ((m == 0) ? sU[SJ] : sU[SM2]));
                const float(*ph)[BX] = ST ? sU[SJ] : ((nz == 1) ? sU[SM] : ((m == nz - 1) ? sU[SM2] : sU[SJ]));
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
        if (o_pt && (ST || (kf >= z0 && kf < z1))) {
            const float w = sW[WK][ty][tx];
            const float lx = sW[WK][ty][xl] + sW[WK][ty][xh] - 2.0f * w;
            const float ly = sW[WK][yl][tx] + sW[WK][yh][tx] - 2.0f * w;
            float lap = lx + ly;
            if (THREE) {
                const float wlo = ST ? wc : ((nz == 1) ? w : ((kf == 0) ? wa : wc));       // mirrored W(k-1)
                const float whi = ST ? wa : ((nz == 1) ? w : ((kf == nz - 1) ? wc : wa));  // mirrored W(k+1)
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

}  // namespace

D4Plan d4_stream_plan(const Dims& d) {
    if (d4_pair_applies(d)) return d4_pair_plan(d);
    D4Plan T;
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
    if (T.pair) return d4_pair_step(T, cur, nxt, f, lam, tau, isg2, d, ctl, check, partials, s);
    const bool three = d.nz > 1;
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
