// Fourth-order diffusion iteration as a 2.5D streaming stencil (2D images are
// the nz == 1 case).  Reference arithmetic: Diffus4th_order_core.c:103-265.
//
// The update needs the weighted Laplacian W at the voxel and its mirrored
// neighbours; W needs U on the mirrored 19-point neighbourhood.  A CTA of
// 32 x 16 threads holds an overlapping tile (thread (tx, ty) on voxel
// (x0 - 2 + tx, y0 - 2 + ty)); W is formed on the inner 30 x 14 voxels, the
// update on the inner 28 x 12.  Step j of each thread:
//   B. publishes U(j) into a four-plane shared-memory ring;
//   A. after the barrier, forms W(j-1) once per voxel from planes j-2, j-1, j
//      of the ring (mirrored in all three axes) into shared memory;
//   C. updates plane j-2 from W of planes j-3, j-2, j-1 (z from registers,
//      x/y from shared memory).
// One barrier per plane.  HBM traffic: read U and f, write U (12 B/voxel);
// the reference's two sweeps move 24 B and store W.
#include "diff4th_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 4, OY = BY - 4;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <bool THREE>
__global__ void __launch_bounds__(NT, 2) k_d4_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                     const float* __restrict__ F, float lam, float tau, float isg2,
                                                     Dims d, int zc, const StopCtl* ctl, int check,
                                                     double2* partials) {
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
    const long long col = in_xy ? ((long long)y * nx + x) : 0;
    auto ld = [&](const float* p, int k) -> float {
        return (in_xy && k >= 0 && k < nz) ? __ldg(p + (long long)k * d.sxy + col) : 0.f;
    };
    auto ring = [](int k) { return (k + 4) & 3; };

    float wa = 0.f, wb = 0.f, wc = 0.f;  // W of planes j-1, j-2, j-3 at this voxel
    float pa = 0.f, pb = 0.f;
    sU[ring(z0 - 2)][ty][tx] = ld(U, z0 - 2);
    sU[ring(z0 - 1)][ty][tx] = ld(U, z0 - 1);
    float uj = ld(U, z0);
    float fa = o_pt ? ld(F, z0 - 2) : 0.f, fb = o_pt ? ld(F, z0 - 1) : 0.f;  // f of planes j-2, j-1

    for (int j = z0; j <= z1 + 1; ++j) {
        const float un1 = (j + 1 <= z1 + 1) ? ld(U, j + 1) : 0.f;  // prefetch U(j+1)
        const float fn = o_pt ? ld(F, j) : 0.f;                      // prefetch f(j)
        // B. publish U(j)
        sU[ring(j)][ty][tx] = uj;
        __syncthreads();
        // A. weighted Laplacian of plane m = j-1 (Diffus4th_order_core.c:176-235)
        const int m = j - 1;
        wc = wb;
        wb = wa;
        wa = 0.f;
        if (m >= 0 && m < nz && m >= z0 - 1 && m <= z1 && w_pt) {
            const int s0 = ring(m);
            const float c0 = sU[s0][ty][tx];
            const float um_x = sU[s0][ty][xl], up_x = sU[s0][ty][xh];
            const float um_y = sU[s0][yl][tx], up_y = sU[s0][yh][tx];
            const float gx = 0.5f * (um_x - up_x), gy = 0.5f * (um_y - up_y);
            const float gx2 = gx * gx, gy2 = gy * gy;
            const float gxx = um_x + up_x - 2.0f * c0;
            const float gyy = um_y + up_y - 2.0f * c0;
            const float gxy = 0.25f * (sU[s0][yl][xl] + sU[s0][yh][xh] - sU[s0][yh][xl] - sU[s0][yl][xh]);
            const float xy2 = 2.0f * gx * gy * gxy;
            float den, vn, vo;
            if (THREE) {
                const int sl = (nz == 1) ? s0 : ((m == 0) ? ring(m + 1) : ring(m - 1));       // mirrored k-1
                const int sh = (nz == 1) ? s0 : ((m == nz - 1) ? ring(m - 1) : ring(m + 1));  // mirrored k+1
                const float zm = sU[sl][ty][tx], zp = sU[sh][ty][tx];
                const float gz = 0.5f * (zm - zp);
                const float gz2 = gz * gz;
                const float gzz = zm + zp - 2.0f * c0;
                const float gxz = 0.25f * (sU[sl][ty][xl] - sU[sl][ty][xh] - sU[sh][ty][xl] + sU[sh][ty][xh]);
                const float gyz = 0.25f * (sU[sl][yl][tx] - sU[sl][yh][tx] - sU[sh][yl][tx] + sU[sh][yh][tx]);
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
            sW[m & 1][ty][tx] = wa;
        }
        // C. update plane kf = j-2 (Diffus4th_order_core.c:237-265); its W was
        // published in the previous step
        const int kf = j - 2;
        if (o_pt && kf >= z0 && kf < z1) {
            const int sk = kf & 1;
            const float w = sW[sk][ty][tx];
            const float lx = sW[sk][ty][xl] + sW[sk][ty][xh] - 2.0f * w;
            const float ly = sW[sk][yl][tx] + sW[sk][yh][tx] - 2.0f * w;
            float lap = lx + ly;
            if (THREE) {
                const float wlo = (nz == 1) ? w : ((kf == 0) ? wa : wc);        // mirrored W(k-1)
                const float whi = (nz == 1) ? w : ((kf == nz - 1) ? wc : wa);   // mirrored W(k+1)
                lap = lap + (wlo + whi - 2.0f * w);
            }
            const float u = sU[ring(kf)][ty][tx];
            const float un = u + tau * (-lam * lap - (u - fa));
            Un[(long long)kf * d.sxy + col] = un;
            if (check) {
                const float df = un - u;
                pa += df * df;
                pb += un * un;
            }
        }
        uj = un1;
        fa = fb;
        fb = fn;
    }
    if (check) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

}  // namespace

D4Plan d4_stream_plan(const Dims& d) {
    D4Plan T;
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_d4_stream<true>, NT);
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
    if (d.nz > 1)
        k_d4_stream<true><<<T.grid, T.block, 0, s>>>(cur, nxt, f, lam, tau, isg2, d, T.zchunk, ctl, check, partials);
    else
        k_d4_stream<false><<<T.grid, T.block, 0, s>>>(cur, nxt, f, lam, tau, isg2, d, T.zchunk, ctl, check, partials);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace cilreg
