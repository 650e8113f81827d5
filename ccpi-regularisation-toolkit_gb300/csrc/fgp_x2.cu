// FGP-TV iteration with two voxels per thread along x (arithmetic
// FGP_TV_core.c:220-269, projection utils.c:180-213): 3D volumes, 2D images
// (also FGP-dTV, k_fgp_x2_2d) and batches of 3D volumes (k_fgp_x2_batch).
//
// The scheme of k_fgp_stream (R and U formed once per voxel, P of plane k-1
// from U's forward differences one plane behind, two barriers per plane, the
// next plane's inputs loaded one plane ahead into registers) with the work
// of a thread doubled along x, as k_rof_pair does for ROF-TV: each thread
// holds the voxel pair (x, x+1), x even, so that the seven inputs, R, U and
// the outputs move in 8-byte accesses, offsets and loop control serve two
// voxels, and the additions, multiplications and fused multiply-adds of both
// voxels issue as paired FP32 instructions.  The projection's reciprocal
// square roots and anisotropic clips stay per voxel.
//
// It runs on volumes of 2^21 to 2^25 voxels, where k_fgp_stream is bound by
// instruction issue and by the latency of its waves rather than by DRAM (the
// larger ones stage their inputs by tensor copies, fgp_tma.cu): 128^3 18.1
// against 20.8 us per iteration, 256^3 115.7 against 122.6, 320^3 218.6
// against 229.9.
//
// A CTA of 16 x 16 threads holds a 32 x 16 tile with the one-voxel halo of
// k_fgp_stream: U on points 1..31, P written on the inner 30 x 14 (whole
// pairs but for the first voxel of thread 0 and the second of thread 15).
// Tile x origins are even (x0 = 30 bx - 2).  Needs nx even; arrays off
// 8-byte alignment run the 4-byte instantiation.
#include <stdlib.h>

#include "fgp_tiled.cuh"
#include "pair.cuh"

namespace cilreg {

namespace {

using namespace pair;

constexpr int ROWS = 16;
constexpr int NTP = PX * ROWS, OYP = ROWS - 2;
constexpr int ZCHUNK = 64;

struct X2Args {
    const float* pc[3];
    const float* po[3];
    float* pn[3];
    const float* f;
    float* u;
    float lam, c, multip;
    int nonneg, aniso, write_u, write_p;
    const float* carr;  // momentum from device memory (graph replays): carr[*cbase + coff]
    const int* cbase;
    int coff;
    const float* b[2];  // FGP-dTV (2D kernel): unit gradient of the reference image
};

// One tile (bx, by, bz) of one volume: the whole CTA walks its z chunk and
// returns its threads' FP32 sums of the stopping check (CHECK).
template <bool CHECK, bool ALIGNED>
__device__ __forceinline__ void x2_tile(const X2Args& a, const Dims& d, int zc, int bx, int by, int bz,
                                        float& pa_out, float& pb_out) {
    __shared__ __align__(16) float sR1[ROWS * TW];
    __shared__ __align__(16) float sR2[ROWS * TW];
    __shared__ __align__(16) float sU[2][ROWS * TW];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int X = tile_x0(bx) + 2 * tx;  // x of the pair's first voxel
    const int y = by * OYP - 1 + ty;
    const int z0 = bz * zc;
    const int z1 = min(z0 + zc, nz);
    // both voxels lie in the volume or neither does (nx even, X even)
    const bool in_xy = X >= 0 && X < nx && y >= 0 && y < ny;
    const bool urow = in_xy && ty >= 1;
    const bool ux = urow && tx >= 1;  // U of the first voxel is needed (point 2 tx >= 1)
    const bool prow = urow && ty <= OYP;
    const bool vx = prow && tx >= 1;       // P of the first voxel written
    const bool vy = prow && tx <= PX - 2;  // P of the second voxel written
    const bool xlast = (X + 2 == nx), ylast = (y == ny - 1);
    const int o = ty * TW + 2 * tx;
    const int oxl = max(o - 1, ty * TW);                 // R1 at x-1 of the first voxel (0 outside: loads)
    const int oxh = min(o + 2, ty * TW + TW - 1);        // U at x+1 of the second voxel
    const int oyl = max(ty - 1, 0) * TW + 2 * tx;        // R2 at y-1
    const int oyh = min(ty + 1, ROWS - 1) * TW + 2 * tx;  // U at y+1
    const int col = in_xy ? (y * nx + X) : 0;
    const int sxy = d.sxy;
    const float2 lam2 = splat(a.lam), mp2 = splat(a.multip);
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };

    // prefetch registers for one plane
    float2 c1 = splat(0.f), o1 = splat(0.f), c2 = splat(0.f), o2 = splat(0.f), c3 = splat(0.f), o3 = splat(0.f);
    float2 fv = splat(0.f);
    auto load_plane = [&](int k) {
        if (in_xy && k >= 0 && k < nz) {
            const int v = k * sxy + col;
            c1 = ldg2(a.pc[0] + v);
            o1 = ldg2(a.po[0] + v);
            c2 = ldg2(a.pc[1] + v);
            o2 = ldg2(a.po[1] + v);
            c3 = ldg2(a.pc[2] + v);
            o3 = ldg2(a.po[2] + v);
            fv = ldg2(a.f + v);
        } else {
            c1 = o1 = c2 = o2 = c3 = o3 = fv = splat(0.f);
        }
    };
    float2 r1p = splat(0.f), r2p = splat(0.f), r3p = splat(0.f), up = splat(0.f);
    float2 uo = splat(0.f);
    float2 pa = splat(0.f), pb = splat(0.f);
    const float2 cm = splat(a.carr ? a.carr[*a.cbase + a.coff] : a.c);
    load_plane(z0 - 1);
    for (int k = z0 - 1; k <= z1; ++k) {
        // 1. R of plane k (FGP_TV_core.c:257-269); start loading plane k+1
        const float2 r1 = fma2(cm, sub2(c1, o1), c1);
        const float2 r2 = fma2(cm, sub2(c2, o2), c2);
        const float2 r3 = fma2(cm, sub2(c3, o3), c3);
        const float2 fk = fv;
        if (k < z1) load_plane(k + 1);
        float2 uo_next = splat(0.f);
        if (CHECK && prow && k >= z0 && k < z1) {
            const float* q = a.u + (k * sxy + col);
            uo_next = ALIGNED ? *reinterpret_cast<const float2*>(q) : make_float2(q[0], q[1]);
        }
        st2(sR1 + o, r1);
        st2(sR2 + o, r2);
        __syncthreads();
        // 2. U of plane k = f - lambda div_b R (FGP_TV_core.c:220-236, clamp :129)
        float2 u = splat(0.f);
        if (urow && k >= z0 && k < nz) {
            const float2 r1l = make_float2(sR1[oxl], r1.x);
            const float2 s = sub2(sub2(sub2(add2(add2(r1, r2), r3), r1l), ld2(sR2 + oyl)), r3p);
            u = fma2(neg2(lam2), s, fk);
            if (a.nonneg) u = make_float2(u.x < 0.f ? 0.f : u.x, u.y < 0.f ? 0.f : u.y);
            if (!ux) u.x = 0.f;
        }
        st2(sU[k & 1] + o, u);
        __syncthreads();
        // 3. P^k of plane k-1 (FGP_TV_core.c:237-256, utils.c:180-213)
        const int kp = k - 1;
        if ((vx || vy) && kp >= z0) {
            const int v = kp * sxy + col;
            if (CHECK) {
                const float2 df = sub2(up, uo);
                const float2 dm = make_float2(vx ? df.x : 0.f, vy ? df.y : 0.f);
                const float2 um = make_float2(vx ? up.x : 0.f, vy ? up.y : 0.f);
                pa = fma2(dm, dm, pa);
                pb = fma2(um, um, pb);
            }
            if (a.write_u) store_pair<ALIGNED>(a.u + v, up, vx, vy);
            if (a.write_p) {
                const float* Up = sU[kp & 1];
                float2 g1 = make_float2(up.x - up.y, xlast ? 0.f : up.y - Up[oxh]);
                const float2 g2 = ylast ? splat(0.f) : sub2(up, ld2(Up + oyh));
                const float2 g3 = (kp != nz - 1) ? sub2(up, u) : splat(0.f);
                float2 p1 = fma2(mp2, g1, r1p);
                float2 p2 = fma2(mp2, g2, r2p);
                float2 p3 = fma2(mp2, g3, r3p);
                if (!a.aniso) {
                    const float2 den = fma2(p3, p3, fma2(p2, p2, mul2(p1, p1)));
                    const float2 sq = make_float2((den.x > 1.f) ? rsqrtf(den.x) : 1.f,
                                                  (den.y > 1.f) ? rsqrtf(den.y) : 1.f);
                    p1 = mul2(p1, sq);
                    p2 = mul2(p2, sq);
                    p3 = mul2(p3, sq);
                } else {
                    p1 = make_float2(unit_clip(p1.x), unit_clip(p1.y));
                    p2 = make_float2(unit_clip(p2.x), unit_clip(p2.y));
                    p3 = make_float2(unit_clip(p3.x), unit_clip(p3.y));
                }
                store_pair<ALIGNED>(a.pn[0] + v, p1, vx, vy);
                store_pair<ALIGNED>(a.pn[1] + v, p2, vx, vy);
                store_pair<ALIGNED>(a.pn[2] + v, p3, vx, vy);
            }
        }
        r1p = r1;
        r2p = r2;
        r3p = r3;
        up = u;
        uo = uo_next;
    }
    pa_out = pa.x + pa.y;
    pb_out = pb.x + pb.y;
}

template <bool CHECK, bool ALIGNED>
__global__ void __launch_bounds__(NTP, 4) k_fgp_x2(X2Args a, Dims d, int zc, const StopCtl* ctl,
                                                   double2* partials) {
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    float pa = 0.f, pb = 0.f;
    x2_tile<CHECK, ALIGNED>(a, d, zc, blockIdx.x, blockIdx.y, blockIdx.z, pa, pb);
    if (CHECK) block_pair_partial<NTP>(pa, pb, partials, block_slot());
}

// One 2D iteration (nz == 1) with the tile of x2_tile, without its plane
// pipeline: R of the pair's pixels (FGP_TV_core.c:168-179), U = f - lambda
// div R on the tile less its first row and column (:119-135), then P from
// the forward differences of U and the projection (:137-166, utils.c:180-213)
// on the inner 30 x 14 pixels; two barriers.  DTV: the FGP-dTV iteration,
// R and the gradient of U each taken onto the complement of the reference's
// unit gradient b at the pixel (FGP_dTV_core.c:311-314, 350-356).
// Tile (bx, by) of one image; `wait` runs once f (and b) are loaded and
// returns false when the run has stopped (the tile then does nothing and
// returns false).
template <bool CHECK, bool ALIGNED, bool DTV, class Wait>
__device__ __forceinline__ bool x2_tile_2d(const X2Args& a, const Dims& d, int bx, int by, Wait wait, float& pa_out,
                                           float& pb_out) {
    __shared__ __align__(16) float sR1[ROWS * TW];
    __shared__ __align__(16) float sR2[ROWS * TW];
    __shared__ __align__(16) float sU[ROWS * TW];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int X = tile_x0(bx) + 2 * tx;  // x of the pair's first pixel
    const int y = by * OYP - 1 + ty;
    const bool in_xy = X >= 0 && X < nx && y >= 0 && y < ny;
    const bool urow = in_xy && ty >= 1;
    const bool ux = urow && tx >= 1;
    const bool prow = urow && ty <= OYP;
    const bool vx = prow && tx >= 1;
    const bool vy = prow && tx <= PX - 2;
    const bool xlast = (X + 2 == nx), ylast = (y == ny - 1);
    const int o = ty * TW + 2 * tx;
    const int oxl = max(o - 1, ty * TW);
    const int oxh = min(o + 2, ty * TW + TW - 1);
    const int oyl = max(ty - 1, 0) * TW + 2 * tx;
    const int oyh = min(ty + 1, ROWS - 1) * TW + 2 * tx;
    const int col = in_xy ? (y * nx + X) : 0;
    const float2 lam2 = splat(a.lam), mp2 = splat(a.multip);
    auto ldg2 = [&](const float* p) -> float2 {
        if (ALIGNED) return __ldg(reinterpret_cast<const float2*>(p));
        return make_float2(__ldg(p), __ldg(p + 1));
    };
    const float2 fv = in_xy ? ldg2(a.f + col) : splat(0.f);  // f never changes: loaded before the wait
    float2 b1 = splat(0.f), b2 = splat(0.f);                  // neither does b
    if (DTV && in_xy) {
        b1 = ldg2(a.b[0] + col);
        b2 = ldg2(a.b[1] + col);
    }
    if (!wait()) return false;
    float2 c1 = splat(0.f), o1 = splat(0.f), c2 = splat(0.f), o2 = splat(0.f);
    if (in_xy) {
        c1 = ldg2(a.pc[0] + col);
        o1 = ldg2(a.po[0] + col);
        c2 = ldg2(a.pc[1] + col);
        o2 = ldg2(a.po[1] + col);
    }
    float2 uo = splat(0.f);
    if (CHECK && prow) {
        const float* q = a.u + col;
        uo = ALIGNED ? *reinterpret_cast<const float2*>(q) : make_float2(q[0], q[1]);
    }
    const float2 cm = splat(a.carr ? a.carr[*a.cbase + a.coff] : a.c);
    float2 r1 = fma2(cm, sub2(c1, o1), c1);
    float2 r2 = fma2(cm, sub2(c2, o2), c2);
    if (DTV) {
        const float2 ip = fma2(r2, b2, mul2(r1, b1));
        r1 = fma2(neg2(ip), b1, r1);
        r2 = fma2(neg2(ip), b2, r2);
    }
    st2(sR1 + o, r1);
    st2(sR2 + o, r2);
    __syncthreads();
    float2 u = splat(0.f);
    if (urow) {
        const float2 r1l = make_float2(sR1[oxl], r1.x);
        const float2 s = sub2(sub2(add2(r1, r2), r1l), ld2(sR2 + oyl));
        u = fma2(neg2(lam2), s, fv);
        if (a.nonneg) u = make_float2(u.x < 0.f ? 0.f : u.x, u.y < 0.f ? 0.f : u.y);
        if (!ux) u.x = 0.f;
    }
    st2(sU + o, u);
    __syncthreads();
    float pa = 0.f, pb = 0.f;
    if (vx || vy) {
        if (CHECK) {
            const float2 df = sub2(u, uo);
            const float2 dm = make_float2(vx ? df.x : 0.f, vy ? df.y : 0.f);
            const float2 um = make_float2(vx ? u.x : 0.f, vy ? u.y : 0.f);
            pa = dm.x * dm.x + dm.y * dm.y;
            pb = um.x * um.x + um.y * um.y;
        }
        if (a.write_u) store_pair<ALIGNED>(a.u + col, u, vx, vy);
        if (a.write_p) {
            float2 g1 = make_float2(u.x - u.y, xlast ? 0.f : u.y - sU[oxh]);
            float2 g2 = ylast ? splat(0.f) : sub2(u, ld2(sU + oyh));
            if (DTV) {
                const float2 ip = fma2(g2, b2, mul2(g1, b1));
                g1 = fma2(neg2(ip), b1, g1);
                g2 = fma2(neg2(ip), b2, g2);
            }
            float2 p1 = fma2(mp2, g1, r1);
            float2 p2 = fma2(mp2, g2, r2);
            if (!a.aniso) {
                const float2 den = fma2(p2, p2, mul2(p1, p1));
                const float2 sq = make_float2((den.x > 1.f) ? rsqrtf(den.x) : 1.f,
                                              (den.y > 1.f) ? rsqrtf(den.y) : 1.f);
                p1 = mul2(p1, sq);
                p2 = mul2(p2, sq);
            } else {
                p1 = make_float2(unit_clip(p1.x), unit_clip(p1.y));
                p2 = make_float2(unit_clip(p2.x), unit_clip(p2.y));
            }
            store_pair<ALIGNED>(a.pn[0] + col, p1, vx, vy);
            store_pair<ALIGNED>(a.pn[1] + col, p2, vx, vy);
        }
    }
    pa_out = pa;
    pb_out = pb;
    return true;
}

template <bool CHECK, bool ALIGNED, bool DTV = false>
__global__ void __launch_bounds__(NTP, 8) k_fgp_x2_2d(X2Args a, Dims d, int zc, const StopCtl* ctl,
                                                      double2* partials) {
    float pa = 0.f, pb = 0.f;
    const bool ran = x2_tile_2d<CHECK, ALIGNED, DTV>(a, d, blockIdx.x, blockIdx.y,
                                                    [&]() {
                                                        pdl_wait();  // the previous iteration has completed
                                                        pdl_trigger();
                                                        return !ctl->stop;
                                                    },
                                                    pa, pb);
    if (CHECK && ran) block_pair_partial<NTP>(pa, pb, partials, block_slot());
}

// one iteration `it` of every volume of a batch (8-byte aligned arrays): a
// flat grid over all volumes' tiles, P^j in ring[j mod 3] as in
// k_fgp_stream_batch; a volume of one plane runs the 2D tile, as its single
// call does
template <bool CHECK>
__global__ void __launch_bounds__(NTP, 4) k_fgp_x2_batch(const FgpBatchVol* __restrict__ vols,
                                                         const int* __restrict__ tile_vol, int it, float c,
                                                         int nonneg, int aniso, int write_u, int write_p) {
    const long long t = blockIdx.x;
    const FgpBatchVol& V = vols[tile_vol[t]];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    const int bx = (int)(lt % V.gx);
    const int by = (int)((lt / V.gx) % V.gy);
    const int bz = (int)(lt / ((long long)V.gx * V.gy));
    // the volume's arguments in shared memory: their uses read them there
    // instead of holding eleven pointers in registers
    __shared__ X2Args a;
    __shared__ Dims d;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        for (int q = 0; q < 3; q++) {
            a.pn[q] = V.ring[it % 3][q];
            a.pc[q] = V.ring[(it + 2) % 3][q];
            a.po[q] = V.ring[(it + 1) % 3][q];
        }
        a.f = V.f;
        a.u = V.u;
        a.lam = V.lam;
        a.c = c;
        a.multip = V.multip;
        a.nonneg = nonneg;
        a.aniso = aniso;
        a.write_u = write_u;
        a.write_p = write_p;
        a.carr = nullptr;
        a.cbase = nullptr;
        a.coff = 0;
        a.b[0] = a.b[1] = nullptr;
        d = V.d;
    }
    __syncthreads();
    float pa = 0.f, pb = 0.f;
    if (d.nz == 1)
        x2_tile_2d<CHECK, true, false>(a, d, bx, by, []() { return true; }, pa, pb);
    else
        x2_tile<CHECK, true>(a, d, V.zc, bx, by, bz, pa, pb);
    if (CHECK) block_pair_partial<NTP>(pa, pb, V.partials, lt);
}

using X2Kernel = decltype(&k_fgp_x2<false, true>);

X2Kernel pick(bool check, bool aligned) {
    if (aligned) return check ? k_fgp_x2<true, true> : k_fgp_x2<false, true>;
    return check ? k_fgp_x2<true, false> : k_fgp_x2<false, false>;
}

}  // namespace

bool fgp_x2_batch_usable(const Dims* dims, const float* const* f, float* const* u, int nvol) {
    for (int v = 0; v < nvol; v++)
        if (dims[v].nx % 2 != 0 || dims[v].n >= (1LL << 31) || !host_aligned8(f[v]) || !host_aligned8(u[v]))
            return false;
    return nvol > 0;
}

void fgp_x2_tile_grid(const Dims& d, int zc, int& gx, int& gy, int& gz) {
    gx = tiles_x(d.nx);
    gy = (d.ny + OYP - 1) / OYP;
    gz = (d.nz + zc - 1) / zc;
}

int fgp_x2_batch_step(const FgpBatchVol* d_vols, const int* d_tile_vol, long long ntiles, int it, float c,
                      int nonneg, int aniso, int write_u, int write_p, int check, cudaStream_t s) {
    if (ntiles < 1 || ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", ntiles);
    const dim3 grid((unsigned)ntiles), block(PX, ROWS, 1);
    if (check)
        k_fgp_x2_batch<true><<<grid, block, 0, s>>>(d_vols, d_tile_vol, it, c, nonneg, aniso, write_u, write_p);
    else
        k_fgp_x2_batch<false><<<grid, block, 0, s>>>(d_vols, d_tile_vol, it, c, nonneg, aniso, write_u, write_p);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

TiledPlan fgp_x2_plan(const Dims& d) {
    TiledPlan T;
    // CILREG_FGP_KERNEL=stream (or simple) keeps a one-voxel kernel
    const char* e = getenv("CILREG_FGP_KERNEL");
    // from 2^21 voxels (128^3): below it the one-voxel kernel's wave is as
    // fast (96^3: 11.8 against 13.0 us per iteration)
    if (e && e[0] != '\0' && e[0] != 'x') return T;
    if (d.nz == 1 && d.nx % 2 == 0 && d.n < (1LL << 31)) {
        // 2D: every size (k_fgp_x2_2d)
        T.use = true;
        T.x2 = true;
        T.block = dim3(PX, ROWS, 1);
        T.zchunk = 1;
        T.grid = dim3(tiles_x(d.nx), (d.ny + OYP - 1) / OYP, 1);
        T.nblocks = (long long)T.grid.x * T.grid.y;
        return T;
    }
    if (!(d.nz > 1 && d.nx % 2 == 0 && d.n >= (1LL << 21) && d.n < (1LL << 31))) return T;
    T.use = true;
    T.x2 = true;
    T.block = dim3(PX, ROWS, 1);
    static const int resident = resident_ctas(k_fgp_x2<false, true>, NTP);
    const int gx = tiles_x(d.nx), gy = (d.ny + OYP - 1) / OYP;
    T.zchunk = wave_zchunk((long long)gx * gy, d.nz, resident, 2, ZCHUNK);
    T.grid = dim3(gx, gy, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int fgp_x2_step(const TiledPlan& T, const float* const pc[3], const float* const po[3], float* const pn[3],
                const float* f, float* u, float lam, float c, float multip, int nonneg, int aniso, int write_u,
                int write_p, int check, const Dims& d, const StopCtl* ctl, double2* partials, cudaStream_t s,
                const float* carr, const int* cbase, int coff, const float* const* b) {
    if (b && d.nz != 1) return fail(ERR_ARG, __FILE__, __LINE__, "the two-voxel FGP-dTV iteration is 2D only");
    X2Args a;
    bool aligned = host_aligned8(f) && host_aligned8(u);
    a.b[0] = b ? b[0] : nullptr;
    a.b[1] = b ? b[1] : nullptr;
    if (b) aligned = aligned && host_aligned8(b[0]) && host_aligned8(b[1]);
    for (int i = 0; i < 3; i++) {
        a.pc[i] = pc[i];
        a.po[i] = po[i];
        a.pn[i] = pn[i];
        aligned = aligned && host_aligned8(pc[i]) && host_aligned8(po[i]) && host_aligned8(pn[i]);
    }
    a.f = f;
    a.u = u;
    a.lam = lam;
    a.c = c;
    a.multip = multip;
    a.nonneg = nonneg;
    a.aniso = aniso;
    a.write_u = write_u;
    a.write_p = write_p;
    a.carr = carr;
    a.cbase = cbase;
    a.coff = coff;
    if (d.nz == 1) {
        X2Kernel k;
        if (b) {
            if (aligned) k = check ? k_fgp_x2_2d<true, true, true> : k_fgp_x2_2d<false, true, true>;
            else k = check ? k_fgp_x2_2d<true, false, true> : k_fgp_x2_2d<false, false, true>;
        } else if (aligned) {
            k = check ? k_fgp_x2_2d<true, true> : k_fgp_x2_2d<false, true>;
        } else {
            k = check ? k_fgp_x2_2d<true, false> : k_fgp_x2_2d<false, false>;
        }
        CILREG_CUDA(launch_pdl(k, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
        return OK;
    }
    CILREG_CUDA(launch_pdl(pick(check != 0, aligned), T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
