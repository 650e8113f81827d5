// LLT-ROF iteration with two voxels per thread along x (reference
// arithmetic LLT_ROF_core.c:54-436): 3D volumes and (k_llt_pair2d) 2D images.
//
// The scheme of k_llt_stream (U through a four-plane shared-memory ring; the
// ROF fluxes and the LLT second-difference terms of plane j-1 formed once per
// voxel into two-plane rings; the update of plane j-2 from them, summed in
// the reference's order; one barrier per plane) with the work of a thread
// doubled along x, as k_rof_pair does for ROF-TV: 8-byte accesses of U, f,
// the terms and the output, offsets and loop control shared by two voxels,
// and paired FP32 additions, multiplications and fused multiply-adds.  The
// reciprocal square roots, minmods and the LLT terms' sign copies stay per
// voxel.
//
// Ring planes beyond the volume are loaded from its mirrored planes, so the
// terms of the first and last plane read their k neighbours without a
// select; the update's mirrored k-1 terms at plane 0 and k+1 term at the last
// plane are selects (terms formed from mirrored planes equal the mirrored
// terms only up to rounding).
//
// A CTA of 16 x 16 threads holds a 32 x 16 tile with a two-voxel halo: the
// terms on the inner 30 x 14 points, the update on the inner 28 x 12, whole
// pairs (threads 1..14 of rows 2..13).  Tile x origins are even
// (x0 = 28 bx - 2).  Needs nx even; arrays off 8-byte alignment run the
// 4-byte instantiation.
#include <stdlib.h>

#include "llt.cuh"
#include "pair.cuh"

namespace cilreg {

namespace {

using namespace pair;

constexpr int ROWS = 16;
constexpr int NTP = PX * ROWS, TP = TW * ROWS;
constexpr int OX4 = TW - 4, OY4 = ROWS - 4;
constexpr int ZCHUNK = 64;

__device__ __forceinline__ float2 minmod_sq2(float2 a, float2 b) {
    const float2 m = make_float2(fmaxf(fminf(a.x, b.x), fminf(fmaxf(a.x, b.x), 0.f)),
                                 fmaxf(fminf(a.y, b.y), fminf(fmaxf(a.y, b.y), 0.f)));
    return mul2(m, m);
}

// dp / sqrt(s) per component
__device__ __forceinline__ float2 normalise2(float2 dp, float2 s) {
    return mul2(dp, make_float2(rsqrtf(s.x), rsqrtf(s.y)));
}

// v / (|v| + 1e-12), the second difference over its magnitude (llt_term
// of llt.cu), with the IEEE quotient's value and without its division for
// almost every v: from |v| = 2^-15 on, 1e-12 is below half an ulp of |v|, so
// the rounded denominator is |v| and the quotient exactly +-1; v = +-0 gives
// itself.  Only the other values (below 2^-15, infinite, NaN) divide: a step
// forms the six terms of its pair by sign copies and, when any of them needs
// it, all six by the division (one branch).
__device__ __forceinline__ float llt_sign1(float v) { return (v == 0.0f) ? v : copysignf(1.0f, v); }
__device__ __forceinline__ float2 llt_sign2(float2 v) { return make_float2(llt_sign1(v.x), llt_sign1(v.y)); }
__device__ __forceinline__ bool llt_divides(float v) {
    const float a = fabsf(v);
    return !(a >= 0x1p-15f && a <= 3.4028234664e38f) && a != 0.0f;
}
__device__ __forceinline__ bool llt_divides2(float2 v) { return llt_divides(v.x) | llt_divides(v.y); }
__device__ __forceinline__ float2 llt_quot2(float2 v) {
    return make_float2(v.x / (fabsf(v.x) + 1.0e-12f), v.y / (fabsf(v.y) + 1.0e-12f));
}

template <bool CHECK, bool ALIGNED, int MINB>
__global__ void __launch_bounds__(NTP, MINB)
    k_llt_pair(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam_rof,
               float lam_llt, float tau, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    __shared__ __align__(16) float sU[4][TP];
    __shared__ __align__(16) float sR1[2][TP];  // ROF D1 (j axis), read at j-1
    __shared__ __align__(16) float sR2[2][TP];  // ROF D2 (i axis), read at i-1
    __shared__ __align__(16) float sL1[2][TP];  // LLT i term, read at i+-1
    __shared__ __align__(16) float sL2[2][TP];  // LLT j term, read at j+-1
    if (ctl->stop) return;
    const float2 EPS2 = splat(1.0e-12f), MTWO2 = splat(-2.0f);
    const float2 tau2 = splat(tau), lrof2 = splat(lam_rof), mlllt2 = splat(-lam_llt);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int X = blockIdx.x * OX4 - 2 + 2 * tx;  // x of the pair's first voxel
    const int y = blockIdx.y * OY4 - 2 + ty;
    const bool upd = tx >= 1 && tx <= PX - 2 && ty >= 2 && ty <= ROWS - 3 && X >= 0 && X < nx && y >= 0 && y < ny;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    // offsets of the first voxel's lower and the second voxel's upper x
    // neighbour: mirrored at the volume edge (LLT_ROF_core.c:115-118),
    // clamped to the tile elsewhere
    const int dxl = ((X == 0) ? o + 1 : max(o - 1, rowlo)) - o;
    const int dxh = ((X + 2 == nx) ? o : min(o + 2, rowhi)) - o;
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
    // (x-1, x) and (x+1, x+2) of the pair at offset `of` of plane `pl`
    auto lo_of = [&](const float* pl, int of, float2 c) { return make_float2(pl[of + dxl], c.x); };
    auto hi_of = [&](const float* pl, int of, float2 c) { return make_float2(c.y, pl[of + dxh]); };

    // ROF D3 and the LLT z term of planes j-1 (a), j-2 (b), j-3 (c)
    float2 r3a = splat(0.f), r3b = splat(0.f), r3c = splat(0.f);
    float2 l3a = splat(0.f), l3b = splat(0.f), l3c = splat(0.f);
    float2 pa = splat(0.f), pb = splat(0.f);
    // U ring slot of plane p: (p - z0 + 4) & 3; term slot: (p - z0 + 2) & 1
    st2(sU[2] + o, ld_u(z0 - 2));
    st2(sU[3] + o, ld_u(z0 - 1));
    float2 uj = ld_u(z0);
    float2 fa = splat(0.f), fb = splat(0.f);

    auto step = [&](auto rr, auto full, auto first, int j) {
        constexpr int R = decltype(rr)::value;
        constexpr bool FULL = decltype(full)::value;
        constexpr bool FIRST = decltype(first)::value;
        constexpr int SJ = R, SM = (R + 3) & 3, SM2 = (R + 2) & 3;  // U slots of planes j, j-1, j-2
        constexpr int WM = (R + 1) & 1, WK = R & 1;                 // term slots of planes j-1, j-2
        const float2 un1 = ld_u(j + 1);
        const float2 fn = ldg2(F + (min(j, nz - 1) * sxy + col));
        // B. publish U(j)
        st2(sU[SJ] + o, uj);
        __syncthreads();
        // A. terms of plane j-1 (LLT_ROF_core.c:104-152, 200-266)
        {
            const float* Um = sU[SM];
            const float2 c = ld2(Um + o);
            const float2 ulo = ld2(sU[SM2] + o), uhi = ld2(sU[SJ] + o);
            const float2 cl = lo_of(Um, o, c), ch = hi_of(Um, o, c);
            const float2 xp = sub2(ch, c), xm = sub2(c, cl);
            const float2 uyh = ld2(Um + oyh), uyl = ld2(Um + oyl);
            const float2 yp = sub2(uyh, c), ym = sub2(c, uyl);
            const float2 zp = sub2(uhi, c), zm = sub2(c, ulo);
            const float2 mx2 = minmod_sq2(xp, xm), my2 = minmod_sq2(yp, ym), mz2 = minmod_sq2(zp, zm);
            const float2 n1 = normalise2(yp, add2(add2(fma2(yp, yp, mx2), mz2), EPS2));
            const float2 n2 = normalise2(xp, add2(add2(fma2(xp, xp, my2), mz2), EPS2));
            const float2 n3 = normalise2(zp, add2(add2(fma2(zp, zp, my2), mx2), EPS2));
            const float2 v3 = add2(fma2(MTWO2, c, uhi), ulo);
            const float2 v1 = add2(fma2(MTWO2, c, ch), cl);
            const float2 v2 = add2(fma2(MTWO2, c, uyh), uyl);
            float2 t3 = llt_sign2(v3), t1 = llt_sign2(v1), t2 = llt_sign2(v2);
            if (llt_divides2(v3) | llt_divides2(v1) | llt_divides2(v2)) {
                t3 = llt_quot2(v3);
                t1 = llt_quot2(v1);
                t2 = llt_quot2(v2);
            }
            l3c = l3b;
            l3b = l3a;
            l3a = t3;
            r3c = r3b;
            r3b = r3a;
            r3a = n3;
            st2(sR1[WM] + o, n1);
            st2(sR2[WM] + o, n2);
            st2(sL1[WM] + o, t1);
            st2(sL2[WM] + o, t2);
        }
        // C. update plane kf = j-2 (LLT_ROF_core.c:404-436); its terms were
        // published in the previous step
        if (FULL) {
            const int kf = j - 2;
            const float* L1 = sL1[WK];
            const float* L2 = sL2[WK];
            const float2 w1 = ld2(L1 + o), w2 = ld2(L2 + o);
            const float2 dxx = add2(fma2(MTWO2, w1, hi_of(L1, o, w1)), lo_of(L1, o, w1));
            const float2 dyy = add2(fma2(MTWO2, w2, ld2(L2 + oyh)), ld2(L2 + oyl));
            const float2 r1 = ld2(sR1[WK] + o), r2 = ld2(sR2[WK] + o);
            const float2 dv1 = sub2(r1, ld2(sR1[WK] + oyl));
            const float2 dv2 = sub2(r2, lo_of(sR2[WK], o, r2));
            // mirrored k-1 terms at plane 0, k+1 term at the last plane
            const float2 llo = (FIRST && kf == 0) ? l3a : l3c;
            const float2 lhi = (kf == nz - 1) ? l3c : l3a;
            const float2 rlo = (FIRST && kf == 0) ? r3a : r3c;
            const float2 dzz = add2(fma2(MTWO2, l3b, lhi), llo);
            const float2 laplc = add2(add2(dxx, dyy), dzz);
            const float2 div = add2(add2(dv1, dv2), sub2(r3b, rlo));
            const float2 u = ld2(sU[SM2] + o);
            const float2 t = sub2(fma2(mlllt2, laplc, mul2(lrof2, div)), sub2(u, fa));
            const float2 un = fma2(tau2, t, u);
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
// CTA is loaded once, the ROF and LLT terms are formed on the inner 30 x 14
// pixels into shared memory, the update on the inner 28 x 12
// (LLT_ROF_core.c:104-152, 200-266, 404-436 in 2D).  Two barriers, no plane
// loop.
constexpr int ROWS2 = 16;
constexpr int NTP2 = PX * ROWS2, TP2 = TW * ROWS2, OY2 = ROWS2 - 4;

template <bool CHECK, bool ALIGNED>
__global__ void __launch_bounds__(NTP2, 6)
    k_llt_pair2d(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam_rof,
                 float lam_llt, float tau, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    __shared__ __align__(16) float sU[TP2];
    __shared__ __align__(16) float sR1[TP2];  // ROF D1 (j axis), read at j-1
    __shared__ __align__(16) float sR2[TP2];  // ROF D2 (i axis), read at i-1
    __shared__ __align__(16) float sL1[TP2];  // LLT i term, read at i+-1
    __shared__ __align__(16) float sL2[TP2];  // LLT j term, read at j+-1
    const float2 EPS2 = splat(1.0e-12f), MTWO2 = splat(-2.0f);
    const float2 tau2 = splat(tau), lrof2 = splat(lam_rof), mlllt2 = splat(-lam_llt);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int X = blockIdx.x * OX4 - 2 + 2 * tx;  // x of the pair's first pixel
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
    auto lo_of = [&](const float* pl, float2 c) { return make_float2(pl[o + dxl], c.x); };
    auto hi_of = [&](const float* pl, float2 c) { return make_float2(c.y, pl[o + dxh]); };
    const float2 fv = ldg2(F + col);  // f never changes during a run: loaded before the wait
    pdl_wait();                       // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    const float2 c = ldg2(U + col);
    st2(sU + o, c);
    __syncthreads();
    {
        const float2 cl = lo_of(sU, c), ch = hi_of(sU, c);
        const float2 xp = sub2(ch, c), xm = sub2(c, cl);
        const float2 uyh = ld2(sU + oyh), uyl = ld2(sU + oyl);
        const float2 yp = sub2(uyh, c), ym = sub2(c, uyl);
        const float2 mx2 = minmod_sq2(xp, xm), my2 = minmod_sq2(yp, ym);
        st2(sR1 + o, normalise2(yp, add2(fma2(yp, yp, mx2), EPS2)));
        st2(sR2 + o, normalise2(xp, add2(fma2(xp, xp, my2), EPS2)));
        const float2 v1 = add2(fma2(MTWO2, c, ch), cl);
        const float2 v2 = add2(fma2(MTWO2, c, uyh), uyl);
        float2 t1 = llt_sign2(v1), t2 = llt_sign2(v2);
        if (llt_divides2(v1) | llt_divides2(v2)) {
            t1 = llt_quot2(v1);
            t2 = llt_quot2(v2);
        }
        st2(sL1 + o, t1);
        st2(sL2 + o, t2);
    }
    __syncthreads();
    float pa = 0.f, pb = 0.f;
    if (upd) {
        const float2 w1 = ld2(sL1 + o), w2 = ld2(sL2 + o);
        const float2 dxx = add2(fma2(MTWO2, w1, hi_of(sL1, w1)), lo_of(sL1, w1));
        const float2 dyy = add2(fma2(MTWO2, w2, ld2(sL2 + oyh)), ld2(sL2 + oyl));
        const float2 r1 = ld2(sR1 + o), r2 = ld2(sR2 + o);
        const float2 dv1 = sub2(r1, ld2(sR1 + oyl));
        const float2 dv2 = sub2(r2, lo_of(sR2, r2));
        const float2 laplc = add2(dxx, dyy);
        const float2 div = add2(dv1, dv2);
        const float2 t = sub2(fma2(mlllt2, laplc, mul2(lrof2, div)), sub2(c, fv));
        const float2 un = fma2(tau2, t, c);
        float* dst = Un + col;
        if (ALIGNED) {
            st2(dst, un);
        } else {
            dst[0] = un.x;
            dst[1] = un.y;
        }
        if (CHECK) {
            const float2 df = sub2(un, c);
            pa = df.x * df.x + df.y * df.y;
            pb = un.x * un.x + un.y * un.y;
        }
    }
    if (CHECK) block_pair_partial<NTP2>(pa, pb, partials, block_slot());
}

// four CTAs per SM at 64 registers (small spills): 0.879 ms per 512^3
// iteration; a 16 x 32 CTA, two per SM, ran 0.882 ms, and three CTAs at 80
// registers without spills 0.996 ms (against 0.933 ms, both before the sign
// shortcut of llt_term1)
constexpr int MINB = 4;
using PairKernel = decltype(&k_llt_pair<false, true, MINB>);

PairKernel pick2d(bool check, bool aligned) {
    if (aligned) return check ? k_llt_pair2d<true, true> : k_llt_pair2d<false, true>;
    return check ? k_llt_pair2d<true, false> : k_llt_pair2d<false, false>;
}

PairKernel pick(bool check, bool aligned) {
    if (aligned) return check ? k_llt_pair<true, true, MINB> : k_llt_pair<false, true, MINB>;
    return check ? k_llt_pair<true, false, MINB> : k_llt_pair<false, false, MINB>;
}

}  // namespace

bool llt_pair_applies(const Dims& d) {
    // CILREG_LLT_KERNEL=stream keeps the one-voxel kernel
    const char* e = getenv("CILREG_LLT_KERNEL");
    return d.nx % 2 == 0 && d.n < (1LL << 31) && !(e && e[0] != '\0' && e[0] != 'p');
}

LltPlan llt_pair_plan(const Dims& d) {
    LltPlan T;
    T.pair = true;
    if (d.nz == 1) {
        T.block = dim3(PX, ROWS2, 1);
        T.zchunk = 1;
        T.grid = dim3((d.nx + OX4 - 1) / OX4, (d.ny + OY2 - 1) / OY2, 1);
        T.nblocks = (long long)T.grid.x * T.grid.y;
        return T;
    }
    T.block = dim3(PX, ROWS, 1);
    const int gx = (d.nx + OX4 - 1) / OX4, gy = (d.ny + OY4 - 1) / OY4;
    static const int resident = resident_ctas(pick(false, true), NTP);
    T.zchunk = wave_zchunk((long long)gx * gy, d.nz, resident, 2, ZCHUNK);
    T.grid = dim3(gx, gy, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

cudaError_t llt_pair_launch(const LltPlan& T, const float* cur, float* nxt, const float* f, float lam_rof,
                            float lam_llt, float tau, const Dims& d, const StopCtl* ctl, int check,
                            double2* partials, cudaStream_t s) {
    const bool aligned = host_aligned8(cur) && host_aligned8(nxt) && host_aligned8(f);
    return launch_pdl(d.nz == 1 ? pick2d(check != 0, aligned) : pick(check != 0, aligned), T.grid, T.block, 0, s,
                      cur, nxt, f, lam_rof, lam_llt, tau, d, T.zchunk, ctl, partials);
}

}  // namespace cilreg
