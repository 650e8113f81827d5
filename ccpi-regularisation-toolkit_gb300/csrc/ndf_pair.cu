// Linear / non-linear diffusion, 3D iteration with two voxels per thread
// along x (Jacobi order; reference arithmetic Diffusion_core.c:108-413).
//
// The scheme of k_ndf_stream (each face flux formed once, by the voxel below
// the face, and used with both signs; six fluxes summed in the reference's
// order) with the work of a thread doubled along x, as k_rof_pair does for
// ROF-TV: U staged through an 8-plane shared-memory ring by 8-byte
// asynchronous copies issued four planes ahead, the pair's own other voxel
// as its inner x neighbour, paired FP32 additions, multiplications and fused
// multiply-adds for both voxels, 8-byte accesses of U, f, the fluxes and the
// output.  Ring planes beyond the volume hold its mirrored planes, so the
// upper k neighbour of the last plane needs no select.
//
// The lower-face fluxes of the update, each mirrored at the volume's lower
// edge to the voxel's own upper flux (Diffusion_core.c:255-265): the west
// flux of the first voxel is -Fx(x-1), or +Fx(x) at x == 0; of the second,
// -Fx(x) of the first.  A per-thread index and sign select between the two,
// and the sign enters through a fused multiply-add by +-1, which rounds the
// sum exactly as the addition of +-Fx does.  Likewise south.
//
// A CTA of 16 x 16 threads holds a 32 x 16 tile with a one-voxel halo; the
// inner 30 x 14 voxels are updated.  Needs nx even; arrays off 8-byte
// alignment run the 4-byte instantiation.
#include <stdlib.h>

#include "ndf_tiled.cuh"
#include "pair.cuh"
#include "tma_ring.cuh"

namespace cilreg {

namespace {

using tma::cp_async4;
using tma::cp_async8;
using tma::cp_async_commit;
using tma::cp_async_wait;

using namespace pair;

constexpr int ROWS = 16;
constexpr int TH = ROWS, OYP = ROWS - 2, NTP = PX * ROWS, TP = TW * ROWS;
constexpr int AHEAD = 4, RING = 8;
constexpr int ZCHUNK = 64;
constexpr size_t SMEM = sizeof(float) * TP * (RING + 4);  // U ring, Fx and Fy (two planes each)

// flux<PEN> (ndf_tiled.cuh) of both components, the products paired
template <int PEN>
__device__ __forceinline__ float2 flux2(float2 e, float sg, float2 isg2) {
    if (PEN == 0) return e;
    if (PEN == 1) {
        const float2 r = mul2(e, isg2);
        return make_float2((fabsf(e.x) > sg) ? copysignf(1.0f, e.x) : r.x,
                           (fabsf(e.y) > sg) ? copysignf(1.0f, e.y) : r.y);
    }
    if (PEN == 2) {
        const float2 r = mul2(e, isg2);
        const float2 q = fma2(r, r, splat(1.0f));
        return mul2(e, make_float2(__frcp_rn(q.x), __frcp_rn(q.y)));
    }
    if (PEN == 3) {
        const float2 r = mul2(e, isg2);
        const float2 w = fma2(neg2(r), r, splat(1.0f));
        const float2 v = mul2(e, mul2(w, w));
        return make_float2((fabsf(e.x) <= sg) ? v.x : 0.0f, (fabsf(e.y) <= sg) ? v.y : 0.0f);
    }
    if (PEN == 4) return make_float2((fabsf(e.x) > sg) ? 0.0f : e.x, (fabsf(e.y) > sg) ? 0.0f : e.y);
    // PEN == 5
    const float2 r = mul2(e, isg2);
    auto one = [&](float ev, float rv) {
        if (fabsf(ev) <= 2.0f * sg) return (fabsf(ev) > sg) ? copysignf(1.0f, ev) : rv;
        return 0.0f;
    };
    return make_float2(one(e.x, r.x), one(e.y, r.y));
}

template <int PEN, bool CHECK, bool ALIGNED>
__global__ void __launch_bounds__(NTP, 4)
    k_ndf_pair(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam, float sg,
               float isg, float tau, Dims d, int zc, const StopCtl* ctl, double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    extern __shared__ __align__(16) float smem[];
    float* const ring = smem;
    float* const sFx = ring + RING * TP;
    float* const sFy = sFx + 2 * TP;
    if (ctl->stop) return;
    const float2 isg2 = splat(isg), lam2 = splat(lam), tau2 = splat(tau);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int X = tile_x0(blockIdx.x) + 2 * tx;  // x of the pair's first voxel
    const int y = blockIdx.y * OYP - 1 + ty;
    const bool row_upd = ty >= 1 && ty <= TH - 2 && y >= 0 && y < ny;
    const bool vx = row_upd && tx >= 1 && X >= 0 && X < nx;
    const bool vy = row_upd && tx <= PX - 2 && X + 1 >= 0 && X + 1 < nx;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    // upper x neighbour of the second voxel (mirrored at the upper edge)
    const int oxh = (X + 2 == nx) ? o : min(o + 2, rowhi);
    // west flux of the first voxel: -Fx(x-1), or +Fx(x) at x == 0
    const int oxw = (X == 0) ? o : max(o - 1, rowlo);
    const float wsg = (X == 0) ? 1.0f : -1.0f;
    // upper y neighbour row (mirrored at the upper edge; a row of length 1
    // maps to itself) and the south flux: -Fy(y-1), or +Fy(y) at y == 0
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    yh = min(max(yh, 0), TH - 1);
    const int oyh = yh * TW + 2 * tx;
    const int oys = (y == 0) ? o : max(ty - 1, 0) * TW + 2 * tx;
    const float2 ssg2 = splat((y == 0) ? 1.0f : -1.0f);
    const float2 wsg2 = make_float2(wsg, -1.0f);
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
    float2 fa = splat(0.f), fb = splat(0.f);
    float2 fxo = splat(0.f), fzo = splat(0.f), fzoo = splat(0.f);

    // step j: fluxes of plane j-1 through its upper faces, update of plane j-2
    // (FULL); FIRST for the first update of a chunk (the only one that can be
    // of plane 0, whose down flux is mirrored)
    auto step = [&](auto rr, auto full, auto first, int j) {
        const int r = ival(rr);
        const int P = r & 1;  // flux slot of plane j
        constexpr bool FULL = decltype(full)::value;
        constexpr bool FIRST = decltype(first)::value;
        issue(r + 2 + AHEAD, j + AHEAD);
        const float2 fe = ldg2(F + (min(j, nz - 1) * sxy + col));
        cp_async_wait<AHEAD>();  // this thread's copy of plane j has landed
        __syncthreads();         // ... and every thread's, and the fluxes of plane j-2
        const float* Uj = slot_of(r + 2);
        const float* Um = slot_of(r + 1);
        const float* Ua = slot_of(r);
        const float2 ub = ld2(Um + o), uc = ld2(Uj + o), ua = ld2(Ua + o);
        // A. upper-face fluxes of plane j-1 (Diffusion_core.c:245-265)
        const float2 fx = flux2<PEN>(make_float2(ub.y - ub.x, Um[oxh] - ub.y), sg, isg2);
        const float2 fy = flux2<PEN>(sub2(ld2(Um + oyh), ub), sg, isg2);
        const float2 fz = flux2<PEN>(sub2(uc, ub), sg, isg2);
        st2(sFx + (1 - P) * TP + o, fx);
        st2(sFy + (1 - P) * TP + o, fy);
        // C. update plane j-2: e + w + n + s + u + d (Diffusion_core.c:267-281)
        if (FULL) {
            const int kf = j - 2;
            const float* Fxp = sFx + P * TP;
            const float* Fyp = sFy + P * TP;
            float2 sum = fma2(wsg2, make_float2(Fxp[oxw], fxo.x), fxo);
            sum = add2(sum, ld2(Fyp + o));
            sum = fma2(ssg2, ld2(Fyp + oys), sum);
            sum = add2(sum, fzo);
            sum = (FIRST && kf == 0) ? add2(sum, fzo) : sub2(sum, fzoo);
            const float2 t = sub2(ua, fa);
            const float2 un = fma2(tau2, fma2(lam2, sum, neg2(t)), ua);
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
        fb = fe;
        fzoo = fzo;
        fxo = fx;
        fzo = fz;
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

// 2D images: one plane per launch, the same pair arithmetic (the 2D path of
// k_ndf_stream: Diffusion_core.c:140-239).  A CTA of 16 x 16 threads updates
// 30 x 14 pixels; at under 40 registers six CTAs fit on an SM, so a 512^2
// image runs in one wave of CTAs.
template <int PEN, bool CHECK, bool ALIGNED>
__global__ void __launch_bounds__(NTP, 6)
    k_ndf_pair2d(const float* __restrict__ U, float* __restrict__ Un, const float* __restrict__ F, float lam,
                 float sg, float isg, float tau, Dims d, int, const StopCtl* ctl, double2* partials) {
    __shared__ __align__(16) float sU[TP];
    __shared__ __align__(16) float sFx[TP];
    __shared__ __align__(16) float sFy[TP];
    const float2 isg2 = splat(isg), lam2 = splat(lam), tau2 = splat(tau);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int X = tile_x0(blockIdx.x) + 2 * tx;
    const int y = blockIdx.y * OYP - 1 + ty;
    const bool row_upd = ty >= 1 && ty <= TH - 2 && y >= 0 && y < ny;
    const bool vx = row_upd && tx >= 1 && X >= 0 && X < nx;
    const bool vy = row_upd && tx <= PX - 2 && X + 1 >= 0 && X + 1 < nx;
    const int o = ty * TW + 2 * tx;
    const int rowlo = ty * TW, rowhi = rowlo + TW - 1;
    const int oxh = (X + 2 == nx) ? o : min(o + 2, rowhi);
    const int oxw = (X == 0) ? o : max(o - 1, rowlo);
    const float2 wsg2 = make_float2((X == 0) ? 1.0f : -1.0f, -1.0f);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    yh = min(max(yh, 0), TH - 1);
    const int oyh = yh * TW + 2 * tx;
    const int oys = (y == 0) ? o : max(ty - 1, 0) * TW + 2 * tx;
    const float2 ssg2 = splat((y == 0) ? 1.0f : -1.0f);
    const int col = min(max(y, 0), ny - 1) * nx + min(max(X, 0), nx - 2);
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    const float2 fv = ldg2(F + col);  // f never changes during a run: loaded before the wait
    pdl_wait();
    pdl_trigger();
    if (ctl->stop) return;
    const float2 u = ldg2(U + col);
    st2(sU + o, u);
    __syncthreads();
    const float2 fx = flux2<PEN>(make_float2(u.y - u.x, sU[oxh] - u.y), sg, isg2);
    const float2 fy = flux2<PEN>(sub2(ld2(sU + oyh), u), sg, isg2);
    st2(sFx + o, fx);
    st2(sFy + o, fy);
    __syncthreads();
    // e + w + n + s (Diffusion_core.c:160-164)
    float2 sum = fma2(wsg2, make_float2(sFx[oxw], fx.x), fx);
    sum = add2(sum, fy);
    sum = fma2(ssg2, ld2(sFy + oys), sum);
    const float2 t = sub2(u, fv);
    const float2 un = fma2(tau2, fma2(lam2, sum, neg2(t)), u);
    store_pair<ALIGNED>(Un + col, un, vx, vy);
    if (CHECK) {
        const float2 df = sub2(un, u);
        const float2 dm = make_float2(vx ? df.x : 0.f, vy ? df.y : 0.f);
        const float2 um = make_float2(vx ? un.x : 0.f, vy ? un.y : 0.f);
        block_pair_partial<NTP>(dm.x * dm.x + dm.y * dm.y, um.x * um.x + um.y * um.y, partials, block_slot());
    }
}

using PairKernel = decltype(&k_ndf_pair<0, false, true>);

template <int PEN>
PairKernel pick_pen(bool check, bool aligned) {
    if (aligned) return check ? k_ndf_pair<PEN, true, true> : k_ndf_pair<PEN, false, true>;
    return check ? k_ndf_pair<PEN, true, false> : k_ndf_pair<PEN, false, false>;
}

PairKernel pick(int pen, bool check, bool aligned) {
    switch (pen) {
        case 0: return pick_pen<0>(check, aligned);
        case 1: return pick_pen<1>(check, aligned);
        case 2: return pick_pen<2>(check, aligned);
        case 3: return pick_pen<3>(check, aligned);
        case 4: return pick_pen<4>(check, aligned);
        case 5: return pick_pen<5>(check, aligned);
        default: return nullptr;
    }
}

template <int PEN>
PairKernel pick2d_pen(bool check, bool aligned) {
    if (aligned) return check ? k_ndf_pair2d<PEN, true, true> : k_ndf_pair2d<PEN, false, true>;
    return check ? k_ndf_pair2d<PEN, true, false> : k_ndf_pair2d<PEN, false, false>;
}

PairKernel pick2d(int pen, bool check, bool aligned) {
    switch (pen) {
        case 0: return pick2d_pen<0>(check, aligned);
        case 1: return pick2d_pen<1>(check, aligned);
        case 2: return pick2d_pen<2>(check, aligned);
        case 3: return pick2d_pen<3>(check, aligned);
        case 4: return pick2d_pen<4>(check, aligned);
        case 5: return pick2d_pen<5>(check, aligned);
        default: return nullptr;
    }
}

// raise the dynamic shared-memory limit of every instantiation once
bool smem_ready() {
    static const bool ok = [] {
        bool r = true;
        for (int p = 0; p <= 5; p++)
            for (int c = 0; c < 2; c++)
                for (int a = 0; a < 2; a++)
                    r = r && cudaFuncSetAttribute(pick(p, c, a), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)SMEM) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    return ok;
}

}  // namespace

bool ndf_pair_applies(const Dims& d) {
    // CILREG_NDF_KERNEL=stream (or simple) keeps a one-voxel kernel
    const char* e = getenv("CILREG_NDF_KERNEL");
    return d.nx % 2 == 0 && d.n < (1LL << 31) && !(e && e[0] != '\0' && e[0] != 'p');
}

NdfPlan ndf_pair_plan(const Dims& d) {
    NdfPlan T;
    T.use = true;
    T.pair = true;
    if (d.nz == 1) {
        T.block = dim3(PX, ROWS, 1);
        T.zchunk = 1;
        T.grid = dim3(tiles_x(d.nx), (d.ny + OYP - 1) / OYP, 1);
        T.nblocks = (long long)T.grid.x * T.grid.y;
        return T;
    }
    T.block = dim3(PX, ROWS, 1);
    const int gx = tiles_x(d.nx), gy = (d.ny + OYP - 1) / OYP;
    int resident = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_ndf_pair<1, false, true>, NTP, SMEM) !=
            cudaSuccess ||
        resident <= 0)
        resident = 1;
    cudaGetLastError();
    T.zchunk = wave_zchunk((long long)gx * gy, d.nz, resident, 2, ZCHUNK);
    T.grid = dim3(gx, gy, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int ndf_pair_step(const NdfPlan& T, int pen, const float* cur, float* nxt, const float* f, float lam, float sg,
                  float isg, float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials,
                  cudaStream_t s) {
    if (pen < 0 || pen > 5) return fail(ERR_ARG, __FILE__, __LINE__, "penalty %d out of range", pen);
    if (d.nz == 1) {
        const bool al = host_aligned8(cur) && host_aligned8(nxt) && host_aligned8(f);
        CILREG_CUDA(launch_pdl(pick2d(pen, check != 0, al), T.grid, T.block, 0, s, cur, nxt, f, lam, sg, isg, tau, d,
                               1, ctl, partials));
        return OK;
    }
    if (!smem_ready())
        return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_ndf_pair");
    const bool aligned = host_aligned8(cur) && host_aligned8(nxt) && host_aligned8(f);
    CILREG_CUDA(launch_pdl(pick(pen, check != 0, aligned), T.grid, T.block, SMEM, s, cur, nxt, f, lam, sg, isg, tau,
                           d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
