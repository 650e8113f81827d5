// ROF-TV 3D iteration with two voxels per thread along x.
//
// The same 2.5D streaming scheme and arithmetic as k_rof_async
// (ROF_TV_core.c:102-317): U staged through an 8-plane shared-memory ring by
// per-thread asynchronous copies issued four planes ahead, fluxes of plane
// j-1 formed while plane j-2 is updated, one barrier per plane.  What
// changes is the work of a thread: it holds the voxel pair (x, x+1), x even,
// so that
//   * every access of a pair (ring planes, the i-neighbour rows, the fluxes,
//     f, lambda, the output) is one 8-byte load or store;
//   * the offsets, plane selects and loop control are shared by two voxels;
//   * the additions, multiplications and fused multiply-adds of both voxels
//     issue as one paired FP32 instruction (FADD2/FMUL2/FFMA2 of sm_100 and
//     later), each rounding exactly as its scalar counterpart.
// The j-axis neighbours of the pair are the pair's own other voxel and one
// scalar load on each side.  Ring planes beyond the volume hold its mirrored
// planes, so the k neighbours of the first and last plane need no select.
// Per voxel this executes about 40% fewer instructions than k_rof_async; the
// iterates agree with it to within a few units in the last place (the
// one-voxel kernel's compiler-contracted multiply-adds are not all the ones
// written out here).
//
// A CTA of 16 x 16 threads holds a 32 x 16 tile with a one-voxel halo; the
// inner 30 x 14 voxels are updated.  Tile x origins are even (x0 = 30 bx - 2)
// so that the pairs of a tile are the pairs of the volume; the kernel needs
// nx even, and 8-byte aligned arrays for its 8-byte accesses (ALIGNED; the
// other instantiation issues two 4-byte accesses instead).
#include <stdlib.h>

#include <type_traits>

#include "rof_tiled.cuh"
#include "pair.cuh"
#include "tma_ring.cuh"

namespace cilreg {

namespace {

using tma::cp_async4;
using tma::cp_async8;
using tma::cp_async_commit;
using tma::cp_async_wait;

using namespace pair;

constexpr int AHEAD = 4, RING = 8;
constexpr int ZCHUNK = 64;

// a tile of TW x ROWS points, one thread row per point row
template <int ROWS>
struct Geo {
    static constexpr int TH = ROWS, OYP = ROWS - 2, NTP = PX * ROWS, TP = TW * ROWS;
    static constexpr int MINB = 64 / ROWS;  // CTAs per SM at 64 registers
    static constexpr size_t SMEM = sizeof(float) * TP * (RING + 4);  // U ring, D1 and D2 (two planes each)
};

// square of minmod(a, b) per component (ROF_TV_core.c:132): the median of a,
// b and 0 has its magnitude
__device__ __forceinline__ float2 minmod_sq2(float2 a, float2 b) {
    const float2 m = make_float2(fmaxf(fminf(a.x, b.x), fminf(fmaxf(a.x, b.x), 0.f)),
                                 fmaxf(fminf(a.y, b.y), fminf(fmaxf(a.y, b.y), 0.f)));
    return mul2(m, m);
}

// dp / sqrt(s) per component, one reciprocal square root each
__device__ __forceinline__ float2 normalise2(float2 dp, float2 s) {
    return mul2(dp, make_float2(rsqrtf(s.x), rsqrtf(s.y)));
}

__device__ __forceinline__ float2 ld2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void st2(float* p, float2 v) { *reinterpret_cast<float2*>(p) = v; }

template <bool CHECK, bool LARR, bool ALIGNED, int ROWS>
__global__ void __launch_bounds__(Geo<ROWS>::NTP, Geo<ROWS>::MINB)
    k_rof_pair(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F,
               const float* __restrict__ lam_arr, float lam, float tau, Dims d, int zc, const StopCtl* ctl,
               double2* partials) {
    constexpr int TH = Geo<ROWS>::TH, OYP = Geo<ROWS>::OYP, NTP = Geo<ROWS>::NTP, TP = Geo<ROWS>::TP;
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    extern __shared__ __align__(16) float smem[];
    float* const ring = smem;
    float* const sD1 = ring + RING * TP;
    float* const sD2 = sD1 + 2 * TP;
    if (ctl->stop) return;
    const float2 EPS2 = splat(1.0e-8f);
    const float2 tau2 = splat(tau);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int X = tile_x0(blockIdx.x) + 2 * tx;  // x of the pair's first voxel
    const int y = blockIdx.y * OYP - 1 + ty;
    const bool row_upd = ty >= 1 && ty <= TH - 2 && y >= 0 && y < ny;
    const bool vx = row_upd && tx >= 1 && X >= 0 && X < nx;           // first voxel updated
    const bool vy = row_upd && tx <= PX - 2 && X + 1 >= 0 && X + 1 < nx;  // second voxel updated
    const int o = ty * TW + 2 * tx;  // the pair's first point in a tile plane
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    // left neighbour of the first voxel and right neighbour of the second:
    // mirrored at the volume edge (ROF_TV_core.c:113-116), clamped to the tile
    // elsewhere (a clamped neighbour only feeds fluxes that no update reads).
    // The first voxel's lower flux D2(x-1) sits at the same index.
    const int oxl = (X == 0) ? o + 1 : max(o - 1, rowlo);
    const int oxh = (X + 2 == nx) ? o : min(o + 2, rowhi);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    yh = min(max(yh, 0), TH - 1);
    yl = min(max(yl, 0), TH - 1);
    const int oyh = yh * TW + 2 * tx, oyl = yl * TW + 2 * tx;
    // pairs outside the volume load the nearest pair inside it
    const int col = min(max(y, 0), ny - 1) * nx + min(max(X, 0), nx - 2);
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const int sxy = d.sxy;
    auto slot_of = [&](int r) -> float* { return ring + (r & (RING - 1)) * TP; };
    auto issue = [&](int r, int k) {
        float* dst = slot_of(r) + o;
        const float* src = U + (ring_plane(k, nz) * sxy + col);
        if (ALIGNED) {
            cp_async8(dst, src);
        } else {
            cp_async4(dst, src);
            cp_async4(dst + 1, src + 1);
        }
        cp_async_commit();
    };
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    float2 pa = splat(0.f), pb = splat(0.f);
    for (int k = z0 - 2; k < z0 + AHEAD; k++) issue(k - z0 + 2, k);
    float2 fa = splat(0.f), la = splat(lam), fb = splat(0.f), lb = splat(lam);
    float2 d1o = splat(0.f), d2o = splat(0.f), d3o = splat(0.f), d3oo = splat(0.f);

    // step j: FULL when plane j-2 is updated, FIRST for the first update of
    // a chunk (the only one that can be of plane 0)
    auto step = [&](auto rr, auto full, auto first, int j) {
        const int r = ival(rr);
        const int P = r & 1;  // flux slot of plane j
        constexpr bool FULL = decltype(full)::value;
        constexpr bool FIRST = decltype(first)::value;
        issue(r + 2 + AHEAD, j + AHEAD);
        const int fo = min(j, nz - 1) * sxy + col;  // f, lambda of plane j (j >= 0)
        const float2 fe = ldg2(F + fo);
        const float2 le = LARR ? ldg2(lam_arr + fo) : splat(lam);
        cp_async_wait<AHEAD>();  // this thread's copy of plane j has landed
        __syncthreads();         // ... and every thread's, and the fluxes of plane j-2
        const float* Uj = slot_of(r + 2);
        const float* Um = slot_of(r + 1);
        const float* Ua = slot_of(r);
        const float2 ub = ld2(Um + o), uc = ld2(Uj + o), ua = ld2(Ua + o);
        // A. fluxes of plane j-1 (its k neighbours ua, uc already mirrored)
        const float dxc = ub.y - ub.x;  // x+1 minus x: forward difference of the first voxel, backward of the second
        const float2 xp = make_float2(dxc, Um[oxh] - ub.y);
        const float2 xm = make_float2(ub.x - Um[oxl], dxc);
        const float2 yp = sub2(ld2(Um + oyh), ub), ym = sub2(ub, ld2(Um + oyl));
        const float2 zp = sub2(uc, ub), zm = sub2(ub, ua);
        const float2 mx2 = minmod_sq2(xp, xm), my2 = minmod_sq2(yp, ym), mz2 = minmod_sq2(zp, zm);
        const float2 n1 = normalise2(yp, add2(add2(fma2(yp, yp, mx2), mz2), EPS2));
        const float2 n2 = normalise2(xp, add2(add2(fma2(xp, xp, my2), mz2), EPS2));
        const float2 n3 = normalise2(zp, add2(add2(fma2(zp, zp, my2), mx2), EPS2));
        st2(sD1 + (1 - P) * TP + o, n1);
        st2(sD2 + (1 - P) * TP + o, n2);
        // C. update plane j-2 (ROF_TV_core.c:269-297): lower fluxes D1(i-1)
        // from the row below, D2(j-1) of the first voxel from the left
        // neighbour and of the second from the first, D3 of plane j-3
        // (mirrored to plane 1 at the first plane)
        if (FULL) {
            const int kf = j - 2;
            const float2 d3lo = (FIRST && kf == 0) ? n3 : d3oo;
            const float2 d1l = ld2(sD1 + P * TP + oyl);
            const float2 d2l = make_float2(sD2[P * TP + oxl], d2o.x);
            const float2 div = add2(add2(sub2(d1o, d1l), sub2(d2o, d2l)), sub2(d3o, d3lo));
            const float2 t = sub2(ua, fa);
            const float2 un = fma2(tau2, fma2(la, div, make_float2(-t.x, -t.y)), ua);
            store_pair<ALIGNED>(Un + (kf * sxy + col), un, vx, vy);
            if (CHECK) {
                const float2 df = sub2(un, ua);
                const float2 dm = make_float2(vx ? df.x : 0.f, vy ? df.y : 0.f);
                const float2 um = make_float2(vx ? un.x : 0.f, vy ? un.y : 0.f);
                pa = fma2(dm, dm, pa);
                pb = fma2(um, um, pb);
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
    using T_ = std::true_type;
    using F_ = std::false_type;
    step(Ic<0>{}, F_{}, F_{}, z0);
    step(Ic<1>{}, F_{}, F_{}, z0 + 1);
    step(Ic<2>{}, T_{}, T_{}, z0 + 2);  // z1 >= z0 + 1: plane z0 is updated
    int j = z0 + 3;
    for (; j + 7 <= z1 + 1; j += 8) {
        step(Ic<3>{}, T_{}, F_{}, j);
        step(Ic<4>{}, T_{}, F_{}, j + 1);
        step(Ic<5>{}, T_{}, F_{}, j + 2);
        step(Ic<6>{}, T_{}, F_{}, j + 3);
        step(Ic<7>{}, T_{}, F_{}, j + 4);
        step(Ic<8>{}, T_{}, F_{}, j + 5);
        step(Ic<9>{}, T_{}, F_{}, j + 6);
        step(Ic<10>{}, T_{}, F_{}, j + 7);
    }
    for (; j <= z1 + 1; j++) step(j - z0, T_{}, F_{}, j);
    cp_async_wait<0>();
    if (CHECK) block_pair_partial<NTP>(pa.x + pa.y, pb.x + pb.y, partials, block_slot());
}

// 2D images: one plane per launch, the same pair arithmetic.  A CTA of
// 16 x ROWS2 threads updates 30 x (ROWS2 - 2) pixels: U of the tile into
// shared memory, the fluxes of every point into shared memory, the update of
// the inner points (ROF_TV_core.c:102-160).  At 25-32 registers eight CTAs
// fit on an SM, so a 512^2 image runs in one wave of CTAs.
constexpr int ROWS2 = 16;
constexpr int TP2 = TW * ROWS2, NTP2 = PX * ROWS2;

template <bool CHECK, bool LARR, bool ALIGNED>
__global__ void __launch_bounds__(NTP2, 8)
    k_rof_pair2d(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F,
                 const float* __restrict__ lam_arr, float lam, float tau, Dims d, int, const StopCtl* ctl,
                 double2* partials) {
    __shared__ __align__(16) float sU[TP2];
    __shared__ __align__(16) float sD1[TP2];
    __shared__ __align__(16) float sD2[TP2];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int X = tile_x0(blockIdx.x) + 2 * tx;
    const int y = blockIdx.y * (ROWS2 - 2) - 1 + ty;
    const bool row_upd = ty >= 1 && ty <= ROWS2 - 2 && y >= 0 && y < ny;
    const bool vx = row_upd && tx >= 1 && X >= 0 && X < nx;
    const bool vy = row_upd && tx <= PX - 2 && X + 1 >= 0 && X + 1 < nx;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    const int oxl = (X == 0) ? o + 1 : max(o - 1, rowlo);
    const int oxh = (X + 2 == nx) ? o : min(o + 2, rowhi);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    int yl = (ny == 1) ? ty : ((y - 1 < 0) ? ty + 1 : ty - 1);
    yh = min(max(yh, 0), ROWS2 - 1);
    yl = min(max(yl, 0), ROWS2 - 1);
    const int oyh = yh * TW + 2 * tx, oyl = yl * TW + 2 * tx;
    const int col = min(max(y, 0), ny - 1) * nx + min(max(X, 0), nx - 2);
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    // f and the lambda map never change during a run: loaded before waiting
    // for the previous iteration (launch_pdl)
    const float2 fv = ldg2(F + col);
    const float2 lv = LARR ? ldg2(lam_arr + col) : splat(lam);
    pdl_wait();
    pdl_trigger();
    if (ctl->stop) return;
    const float2 u = ldg2(U + col);
    st2(sU + o, u);
    __syncthreads();
    const float dxc = u.y - u.x;
    const float2 xp = make_float2(dxc, sU[oxh] - u.y);
    const float2 xm = make_float2(u.x - sU[oxl], dxc);
    const float2 yp = sub2(ld2(sU + oyh), u), ym = sub2(u, ld2(sU + oyl));
    const float2 mx2 = minmod_sq2(xp, xm), my2 = minmod_sq2(yp, ym);
    const float2 EPS2 = splat(1.0e-8f);
    const float2 d1 = normalise2(yp, add2(fma2(yp, yp, mx2), EPS2));
    const float2 d2 = normalise2(xp, add2(fma2(xp, xp, my2), EPS2));
    st2(sD1 + o, d1);
    st2(sD2 + o, d2);
    __syncthreads();
    const float2 div = add2(sub2(d1, ld2(sD1 + oyl)), sub2(d2, make_float2(sD2[oxl], d2.x)));
    const float2 t = sub2(u, fv);
    const float2 un = fma2(splat(tau), fma2(lv, div, neg2(t)), u);
    store_pair<ALIGNED>(Un + col, un, vx, vy);
    float2 pa = splat(0.f), pb = splat(0.f);
    if (CHECK) {
        const float2 df = sub2(un, u);
        const float2 dm = make_float2(vx ? df.x : 0.f, vy ? df.y : 0.f);
        const float2 um = make_float2(vx ? un.x : 0.f, vy ? un.y : 0.f);
        pa = mul2(dm, dm);
        pb = mul2(um, um);
        block_pair_partial<NTP2>(pa.x + pa.y, pb.x + pb.y, partials, block_slot());
    }
}

// 16 rows: four CTAs per SM (32 warps in four independent barrier groups).
// A 32-row tile has 7% fewer halo voxels but two CTAs per SM, and measured
// 0.475 against 0.436 ms per 512^3 iteration.
constexpr int ROWS = 16;
using PairKernel = decltype(&k_rof_pair<false, false, true, ROWS>);

PairKernel pick(bool check, bool larr, bool aligned) {
    if (aligned)
        return check ? (larr ? k_rof_pair<true, true, true, ROWS> : k_rof_pair<true, false, true, ROWS>)
                     : (larr ? k_rof_pair<false, true, true, ROWS> : k_rof_pair<false, false, true, ROWS>);
    return check ? (larr ? k_rof_pair<true, true, false, ROWS> : k_rof_pair<true, false, false, ROWS>)
                 : (larr ? k_rof_pair<false, true, false, ROWS> : k_rof_pair<false, false, false, ROWS>);
}

PairKernel pick2d(bool check, bool larr, bool aligned) {
    if (aligned)
        return check ? (larr ? k_rof_pair2d<true, true, true> : k_rof_pair2d<true, false, true>)
                     : (larr ? k_rof_pair2d<false, true, true> : k_rof_pair2d<false, false, true>);
    return check ? (larr ? k_rof_pair2d<true, true, false> : k_rof_pair2d<true, false, false>)
                 : (larr ? k_rof_pair2d<false, true, false> : k_rof_pair2d<false, false, false>);
}

// raise the dynamic shared-memory limit of every instantiation once
bool smem_ready() {
    static const bool ok = [] {
        bool r = true;
        for (int c = 0; c < 2; c++)
            for (int l = 0; l < 2; l++)
                for (int a = 0; a < 2; a++)
                    r = r && cudaFuncSetAttribute(pick(c, l, a), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)Geo<ROWS>::SMEM) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    return ok;
}

}  // namespace

bool rof_pair_applies(const Dims& d) {
    // CILREG_ROF_KERNEL=async (or reg, simple) keeps the one-voxel kernels
    const char* ek = getenv("CILREG_ROF_KERNEL");
    return d.nx % 2 == 0 && d.n < (1LL << 31) && !(ek && ek[0] != '\0' && ek[0] != 'p');
}

RofPlan rof_pair_plan(const Dims& d) {
    RofPlan T;
    T.pair = true;
    if (d.nz == 1) {
        T.block = dim3(PX, ROWS2, 1);
        T.zchunk = 1;
        T.grid = dim3(tiles_x(d.nx), (d.ny + ROWS2 - 3) / (ROWS2 - 2), 1);
        T.nblocks = (long long)T.grid.x * T.grid.y;
        return T;
    }
    T.block = dim3(PX, ROWS, 1);
    const int gx = tiles_x(d.nx), gy = (d.ny + Geo<ROWS>::OYP - 1) / Geo<ROWS>::OYP;
    int resident = 0;
    const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &resident, k_rof_pair<false, false, true, ROWS>, Geo<ROWS>::NTP, Geo<ROWS>::SMEM);
    if (e != cudaSuccess || resident <= 0) resident = 1;
    cudaGetLastError();
    T.zchunk = wave_zchunk((long long)gx * gy, d.nz, resident, 2, ZCHUNK);
    T.grid = dim3(gx, gy, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int rof_pair_step(const RofPlan& T, const float* cur, float* nxt, const float* f, const float* lam_arr, float lam,
                  float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials, cudaStream_t s) {
    const bool larr = lam_arr != nullptr;
    const bool aligned =
        host_aligned8(cur) && host_aligned8(nxt) && host_aligned8(f) && (!larr || host_aligned8(lam_arr));
    if (d.nz == 1) {
        CILREG_CUDA(launch_pdl(pick2d(check != 0, larr, aligned), T.grid, T.block, 0, s, cur, nxt, f, lam_arr, lam,
                               tau, d, 1, ctl, partials));
        return OK;
    }
    if (!smem_ready())
        return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_rof_pair");
    CILREG_CUDA(launch_pdl(pick(check != 0, larr, aligned), T.grid, T.block, Geo<ROWS>::SMEM, s, cur, nxt, f,
                           lam_arr, lam, tau, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
