// Fourth-order diffusion iteration with two voxels per thread along x
// (reference arithmetic Diffus4th_order_core.c:103-265): 3D volumes and
// (k_d4_pair2d) 2D images.
//
// The scheme of k_d4_stream (U through a four-plane shared-memory ring, the
// weighted Laplacian W formed once per voxel into a two-plane ring, the
// update from W; one barrier per plane) with the work of a thread doubled
// along x, as k_rof_pair does for ROF-TV: each thread holds the pair
// (x, x+1), x even, so that U, f, W and the output move in 8-byte accesses,
// the offsets and loop control serve two voxels, and the additions,
// multiplications and fused multiply-adds of both voxels issue as paired FP32
// instructions.  The pair's x neighbours x-1 and x+2 are single loads (or,
// at the volume's edge, its own other voxel: the reference's mirror).
//
// Ring planes beyond the volume are loaded from its mirrored planes (plane -1
// from plane 1, plane nz from plane nz-2), so W of the first and last plane
// reads its k neighbours without a select.  The update's mirrored W(k-1) at
// the first plane and W(k+1) at the last one are selects: W formed from
// mirrored planes equals the mirrored W only up to rounding.
//
// The two reciprocals of W (1/den and the diffusivity 1/(1 + den/sigma^2))
// are rcp2's (pair.cuh): the approximate reciprocal with one paired
// Newton-Raphson step, within an ulp of the IEEE reciprocal of the one-voxel
// kernels and much cheaper to issue (0.823 -> 0.707 ms per 512^3 iteration).
//
// A CTA of 16 x ROWS threads holds a 32 x ROWS tile with a two-voxel halo:
// W on the inner 30 x (ROWS-2) points, the update on the inner 28 x (ROWS-4),
// whole pairs (threads 1..14 of rows 2..ROWS-3).  Tile x origins are even
// (x0 = 28 bx - 2).  Needs nx even; arrays off 8-byte alignment run the
// 4-byte instantiation.
#include <stdlib.h>

#include "diff4th_tiled.cuh"
#include "pair.cuh"

namespace cilreg {

namespace {

using namespace pair;

constexpr int OX4 = TW - 4;  // updated voxels along x
constexpr int ZCHUNK = 64;

template <int ROWS>
struct Geo {
    static constexpr int NTP = PX * ROWS, TP = TW * ROWS, OY = ROWS - 4;
    static constexpr int MINB = (ROWS >= 32) ? 2 : 4;
};

// x origin of tile bx (even; the first tile starts two voxels before the volume)
__device__ __forceinline__ int d4_tile_x0(int bx) { return bx * OX4 - 2; }

template <bool CHECK, bool ALIGNED, int ROWS>
__global__ void __launch_bounds__(Geo<ROWS>::NTP, Geo<ROWS>::MINB)
    k_d4_pair(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam,
              float tau, float isg2, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    constexpr int TP = Geo<ROWS>::TP, NTP = Geo<ROWS>::NTP;
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ __align__(16) float sU[4][TP];
    __shared__ __align__(16) float sW[2][TP];
    if (ctl->stop) return;
    const float EPS = 1.0e-7f;
    const float2 ONE2 = splat(1.0f), HALF2 = splat(0.5f), QUART2 = splat(0.25f);
    const float2 TWO2 = splat(2.0f), MTWO2 = splat(-2.0f), isg22 = splat(isg2);
    const float2 tau2 = splat(tau), mlam2 = splat(-lam);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int X = d4_tile_x0(blockIdx.x) + 2 * tx;  // x of the pair's first voxel
    const int y = blockIdx.y * Geo<ROWS>::OY - 2 + ty;
    const bool upd = tx >= 1 && tx <= PX - 2 && ty >= 2 && ty <= ROWS - 3 && X >= 0 && X < nx && y >= 0 && y < ny;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    // x offsets (from the pair's first point) of the first voxel's lower and
    // the second voxel's upper x neighbour: mirrored at the volume edge,
    // clamped to the tile elsewhere (a clamped neighbour feeds only W and
    // updates that are never used)
    const int dxl = ((X == 0) ? o + 1 : max(o - 1, rowlo)) - o;
    const int dxh = ((X + 2 == nx) ? o : min(o + 2, rowhi)) - o;
    // lower and upper y neighbour rows (mirrored; a row of length 1 maps to itself)
    int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    yl = min(max(yl, 0), ROWS - 1);
    yh = min(max(yh, 0), ROWS - 1);
    const int oyl = yl * TW + 2 * tx, oyh = yh * TW + 2 * tx;
    const int col = min(max(y, 0), ny - 1) * nx + min(max(X, 0), nx - 2);
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const int sxy = d.sxy;
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    auto ld_u = [&](int k) -> float2 { return ldg2(U + (ring_plane(k, nz) * sxy + col)); };

    // the pair at offset `of` of a plane with its x neighbours: (x-1, x) and
    // (x+1, x+2) as two pairs
    struct Nb {
        float2 lo, c, hi;
    };
    auto nb = [&](const float* pl, int of) -> Nb {
        const float2 c = ld2(pl + of);
        return {make_float2(pl[of + dxl], c.x), c, make_float2(c.y, pl[of + dxh])};
    };

    float2 wa = splat(0.f), wb = splat(0.f), wc = splat(0.f);  // W of planes j-1, j-2, j-3
    float2 pa = splat(0.f), pb = splat(0.f);
    // U ring slot of plane p: (p - z0 + 4) & 3; W ring slot: (p - z0 + 2) & 1
    st2(sU[2] + o, ld_u(z0 - 2));
    st2(sU[3] + o, ld_u(z0 - 1));
    float2 uj = ld_u(z0);
    float2 fa = splat(0.f), fb = splat(0.f);  // f of planes j-2, j-1

    // step j (R = (j - z0) & 3): publish U(j), form W(j-1), update plane j-2
    // when FULL; FIRST: the chunk's first update (the only one that can be of
    // plane 0)
    auto step = [&](auto rr, auto full, auto first, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr bool FULL = decltype(full)::value;
        constexpr bool FIRST = decltype(first)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // W slots of planes j-1, j-2
        const float2 un1 = ld_u(j + 1);                             // prefetch U(j+1)
        const float2 fn = ldg2(F + (min(j, nz - 1) * sxy + col));  // prefetch f(j)
        // B. publish U(j)
        st2(sU[SJ] + o, uj);
        __syncthreads();
        // A. weighted Laplacian of plane j-1 (Diffus4th_order_core.c:176-235);
        // its k neighbours are planes j-2 and j (mirrored in the ring)
        {
            const float* pm = sU[SM];
            const float* pl = sU[SM2];
            const float* ph = sU[SJ];
            const Nb m0 = nb(pm, o), ml = nb(pm, oyl), mh = nb(pm, oyh);
            const float2 c0 = m0.c;
            const float2 gx = mul2(HALF2, sub2(m0.lo, m0.hi));
            const float2 gy = mul2(HALF2, sub2(ml.c, mh.c));
            const float2 gx2 = mul2(gx, gx), gy2 = mul2(gy, gy);
            const float2 gxx = fma2(MTWO2, c0, add2(m0.lo, m0.hi));
            const float2 gyy = fma2(MTWO2, c0, add2(ml.c, mh.c));
            const float2 gxy = mul2(QUART2, sub2(sub2(add2(ml.lo, mh.hi), mh.lo), ml.hi));
            const float2 xy2 = mul2(mul2(mul2(TWO2, gx), gy), gxy);
            const Nb l0 = nb(pl, o), h0 = nb(ph, o);
            const float2 zm = l0.c, zp = h0.c;
            const float2 gz = mul2(HALF2, sub2(zm, zp));
            const float2 gz2 = mul2(gz, gz);
            const float2 gzz = fma2(MTWO2, c0, add2(zm, zp));
            const float2 gxz = mul2(QUART2, add2(sub2(sub2(l0.lo, l0.hi), h0.lo), h0.hi));
            const float2 gyz =
                mul2(QUART2, add2(sub2(sub2(ld2(pl + oyl), ld2(pl + oyh)), ld2(ph + oyl)), ld2(ph + oyh)));
            const float2 xz2 = mul2(mul2(mul2(TWO2, gx), gz), gxz);
            const float2 yz2 = mul2(mul2(mul2(TWO2, gy), gz), gyz);
            const float2 den = add2(add2(gx2, gy2), gz2);
            float2 nn = fma2(gzz, gz2, fma2(gyy, gy2, mul2(gxx, gx2)));
            nn = add2(add2(add2(nn, xy2), xz2), yz2);
            float2 oo = fma2(add2(gx2, gy2), gzz, fma2(add2(gx2, gz2), gyy, mul2(add2(gy2, gz2), gxx)));
            oo = sub2(sub2(sub2(oo, xy2), xz2), yz2);
            const float2 iq = rcp2(make_float2((den.x <= EPS) ? EPS : den.x, (den.y <= EPS) ? EPS : den.y));
            const float2 vn = mul2(nn, iq), vo = mul2(oo, iq);
            const float2 q = fma2(den, isg22, ONE2);
            const float2 c = rcp2(q);
            wc = wb;
            wb = wa;
            wa = fma2(mul2(c, c), vn, mul2(c, vo));
            st2(sW[WM] + o, wa);
        }
        // C. update plane kf = j-2 (Diffus4th_order_core.c:237-265); its W was
        // published in the previous step
        if (FULL) {
            const int kf = j - 2;
            const Nb w0 = nb(sW[WK], o);
            const float2 w = w0.c;
            const float2 lx = fma2(MTWO2, w, add2(w0.lo, w0.hi));
            const float2 ly = fma2(MTWO2, w, add2(ld2(sW[WK] + oyl), ld2(sW[WK] + oyh)));
            // mirrored W(k-1) at the first plane, W(k+1) at the last
            const float2 wlo = (FIRST && kf == 0) ? wa : wc;
            const float2 whi = (kf == nz - 1) ? wc : wa;
            const float2 lap = add2(add2(lx, ly), fma2(MTWO2, w, add2(wlo, whi)));
            const float2 u = ld2(sU[SM2] + o);
            const float2 un = fma2(tau2, fma2(mlam2, lap, neg2(sub2(u, fa))), u);
            if (upd) {
                float* dst = Un + (kf * sxy + col);
                if (ALIGNED) {
                    st2(dst, un);
                } else {
                    dst[0] = un.x;
                    dst[1] = un.y;
                }
                if (CHECK) {
                    const float2 df = sub2(un, u);
                    pa = fma2(df, df, pa);
                    pb = fma2(un, un, pb);
                }
            }
        }
        uj = un1;
        fa = fb;
        fb = fn;
    };
    using T_ = std::true_type;
    using F_ = std::false_type;
    step(Ic<0>{}, F_{}, F_{}, z0);
    step(Ic<1>{}, F_{}, F_{}, z0 + 1);
    step(Ic<2>{}, T_{}, T_{}, z0 + 2);  // z1 >= z0 + 1: plane z0 is updated
    int j = z0 + 3;
    for (; j + 3 <= z1 + 1; j += 4) {
        step(Ic<3>{}, T_{}, F_{}, j);
        step(Ic<0>{}, T_{}, F_{}, j + 1);
        step(Ic<1>{}, T_{}, F_{}, j + 2);
        step(Ic<2>{}, T_{}, F_{}, j + 3);
    }
    if (j <= z1 + 1) step(Ic<3>{}, T_{}, F_{}, j);
    if (j + 1 <= z1 + 1) step(Ic<0>{}, T_{}, F_{}, j + 1);
    if (j + 2 <= z1 + 1) step(Ic<1>{}, T_{}, F_{}, j + 2);
    if (CHECK) block_pair_partial<NTP>(pa.x + pa.y, pb.x + pb.y, partials, block_slot());
}

// One 2D iteration (nz == 1), two pixels per thread: the pair of a 16 x 16
// CTA is loaded once, W is formed on the inner 30 x 14 pixels into shared
// memory, the update on the inner 28 x 12 (Diffus4th_order_core.c:103-150,
// 237-265).  Two barriers, no plane loop: 256-thread CTAs, several per SM,
// keep a 2D image's short launch latency-tolerant.
constexpr int ROWS2 = 16;
constexpr int NTP2 = PX * ROWS2, TP2 = TW * ROWS2, OY2 = ROWS2 - 4;

template <bool CHECK, bool ALIGNED>
__global__ void __launch_bounds__(NTP2, 6)
    k_d4_pair2d(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam,
                float tau, float isg2, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    __shared__ __align__(16) float sU[TP2];
    __shared__ __align__(16) float sW[TP2];
    const float EPS = 1.0e-7f;
    const float2 HALF2 = splat(0.5f), QUART2 = splat(0.25f), TWO2 = splat(2.0f), MTWO2 = splat(-2.0f);
    const float2 ONE2 = splat(1.0f), isg22 = splat(isg2), tau2 = splat(tau), mlam2 = splat(-lam);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int X = d4_tile_x0(blockIdx.x) + 2 * tx;  // x of the pair's first pixel
    const int y = blockIdx.y * OY2 - 2 + ty;
    const bool upd = tx >= 1 && tx <= PX - 2 && ty >= 2 && ty <= ROWS2 - 3 && X >= 0 && X < nx && y >= 0 && y < ny;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    const int dxl = ((X == 0) ? o + 1 : max(o - 1, rowlo)) - o;
    const int dxh = ((X + 2 == nx) ? o : min(o + 2, rowhi)) - o;
    int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    yl = min(max(yl, 0), ROWS2 - 1);
    yh = min(max(yh, 0), ROWS2 - 1);
    const int oyl = yl * TW + 2 * tx, oyh = yh * TW + 2 * tx;
    const int col = min(max(y, 0), ny - 1) * nx + min(max(X, 0), nx - 2);
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    const float2 fv = ldg2(F + col);  // f never changes during a run: loaded before the wait
    pdl_wait();                       // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    const float2 u = ldg2(U + col);
    st2(sU + o, u);
    __syncthreads();
    {
        const float2 lo = make_float2(sU[o + dxl], u.x), hi = make_float2(u.y, sU[o + dxh]);
        const float2 ml = ld2(sU + oyl), mh = ld2(sU + oyh);
        const float2 mll = make_float2(sU[oyl + dxl], ml.x), mlh = make_float2(ml.y, sU[oyl + dxh]);
        const float2 mhl = make_float2(sU[oyh + dxl], mh.x), mhh = make_float2(mh.y, sU[oyh + dxh]);
        const float2 gx = mul2(HALF2, sub2(lo, hi));
        const float2 gy = mul2(HALF2, sub2(ml, mh));
        const float2 gx2 = mul2(gx, gx), gy2 = mul2(gy, gy);
        const float2 gxx = fma2(MTWO2, u, add2(lo, hi));
        const float2 gyy = fma2(MTWO2, u, add2(ml, mh));
        const float2 gxy = mul2(QUART2, sub2(sub2(add2(mll, mhh), mhl), mlh));
        const float2 xy2 = mul2(mul2(mul2(TWO2, gx), gy), gxy);
        const float2 den = add2(gx2, gy2);
        const float2 nn = fma2(gyy, gy2, fma2(gxx, gx2, xy2));
        const float2 oo = fma2(gyy, gx2, fma2(gxx, gy2, neg2(xy2)));
        const float2 iq = rcp2(make_float2((den.x <= EPS) ? EPS : den.x, (den.y <= EPS) ? EPS : den.y));
        const float2 vn = mul2(nn, iq), vo = mul2(oo, iq);
        const float2 c = rcp2(fma2(den, isg22, ONE2));
        st2(sW + o, fma2(mul2(c, c), vn, mul2(c, vo)));
    }
    __syncthreads();
    float pa = 0.f, pb = 0.f;
    if (upd) {
        const float2 w = ld2(sW + o);
        const float2 lx = fma2(MTWO2, w, add2(make_float2(sW[o + dxl], w.x), make_float2(w.y, sW[o + dxh])));
        const float2 ly = fma2(MTWO2, w, add2(ld2(sW + oyl), ld2(sW + oyh)));
        const float2 lap = add2(lx, ly);
        const float2 un = fma2(tau2, fma2(mlam2, lap, neg2(sub2(u, fv))), u);
        float* dst = Un + col;
        if (ALIGNED) {
            st2(dst, un);
        } else {
            dst[0] = un.x;
            dst[1] = un.y;
        }
        if (CHECK) {
            const float2 df = sub2(un, u);
            pa = df.x * df.x + df.y * df.y;
            pb = un.x * un.x + un.y * un.y;
        }
    }
    if (CHECK) block_pair_partial<NTP2>(pa, pb, partials, block_slot());
}

// 32 rows: two CTAs (32 warps) per SM; 16 rows (four CTAs) measured the same
// at 512^3 (0.824 ms per iteration) and 3% slower at 256^3
constexpr int ROWS = 32;
using PairKernel = decltype(&k_d4_pair<false, true, ROWS>);

PairKernel pick(bool check, bool aligned) {
    if (aligned) return check ? k_d4_pair<true, true, ROWS> : k_d4_pair<false, true, ROWS>;
    return check ? k_d4_pair<true, false, ROWS> : k_d4_pair<false, false, ROWS>;
}

PairKernel pick2d(bool check, bool aligned) {
    if (aligned) return check ? k_d4_pair2d<true, true> : k_d4_pair2d<false, true>;
    return check ? k_d4_pair2d<true, false> : k_d4_pair2d<false, false>;
}

}  // namespace

bool d4_pair_applies(const Dims& d) {
    // CILREG_D4_KERNEL=stream (or simple) keeps a one-voxel kernel
    const char* e = getenv("CILREG_D4_KERNEL");
    return d.nx % 2 == 0 && d.n < (1LL << 31) && !(e && e[0] != '\0' && e[0] != 'p');
}

D4Plan d4_pair_plan(const Dims& d) {
    D4Plan T;
    T.pair = true;
    if (d.nz == 1) {
        T.block = dim3(PX, ROWS2, 1);
        T.zchunk = 1;
        T.grid = dim3((d.nx + OX4 - 1) / OX4, (d.ny + OY2 - 1) / OY2, 1);
        T.nblocks = (long long)T.grid.x * T.grid.y;
        return T;
    }
    T.block = dim3(PX, ROWS, 1);
    const int gx = (d.nx + OX4 - 1) / OX4, gy = (d.ny + Geo<ROWS>::OY - 1) / Geo<ROWS>::OY;
    int resident = 0;
    const cudaError_t e =
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_d4_pair<false, true, ROWS>, Geo<ROWS>::NTP, 0);
    if (e != cudaSuccess || resident <= 0) resident = 1;
    cudaGetLastError();
    T.zchunk = wave_zchunk((long long)gx * gy, d.nz, resident, 2, ZCHUNK);
    T.grid = dim3(gx, gy, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int d4_pair_step(const D4Plan& T, const float* cur, float* nxt, const float* f, float lam, float tau, float isg2,
                 const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    const bool aligned = host_aligned8(cur) && host_aligned8(nxt) && host_aligned8(f);
    CILREG_CUDA(launch_pdl(d.nz == 1 ? pick2d(check != 0, aligned) : pick(check != 0, aligned), T.grid, T.block, 0,
                           s, cur, nxt, f, lam, tau, isg2, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
