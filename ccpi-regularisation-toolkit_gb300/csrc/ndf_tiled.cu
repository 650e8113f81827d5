// Linear / non-linear diffusion iteration as a 2.5D streaming stencil (2D
// images are the nz == 1 case), Jacobi order.  Reference arithmetic:
// Diffusion_core.c:108-413.
//
// The update of a voxel sums the edge-stopping flux of its six mirrored
// neighbour differences.  Each flux is odd in the difference, so the flux
// through the face between two voxels is formed once (by the lower voxel:
// Fx = g(U[i+1] - U[i]), with the mirrored neighbour at the upper edge) and
// the upper voxel uses -Fx.  The lower edge's mirror (w = U[i+1]) makes the
// west flux equal the voxel's own east flux there.  Three flux evaluations per
// voxel instead of six, bit-identical terms.
//
// A CTA of 32 x 16 threads holds a tile with a one-voxel halo (thread (tx, ty)
// on voxel (x0 - 1 + tx, y0 - 1 + ty)); the inner 30 x 14 voxels are updated.
// Step j of each thread, walking a chunk of z planes:
//   A. forms the fluxes of plane j-1 through its upper i, j and k faces (i/j
//      neighbours from shared memory, k neighbour from its registers); the i
//      and j fluxes go to shared memory, all three stay in registers;
//   B. publishes U(j) (loaded two steps earlier) to shared memory;
//   C. updates plane j-2: U += tau (lambda (e + w + n + s + u + d) - (U - f)),
//      summed in the reference's order.
// One barrier per plane, no boundary branches in the loop, ring slots as
// compile-time constants.  HBM traffic: read U and f, write U (12 B/voxel).
#include <string.h>

#include <type_traits>

#include "ndf_tiled.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 2, OY = BY - 2;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

template <int V>
using Ic = std::integral_constant<int, V>;

template <bool THREE, int PEN, bool CHECK>
__global__ void __launch_bounds__(NT, 3) k_ndf_stream(const float* __restrict__ U, float* __restrict__ Un,
                                                      const float* __restrict__ F, float lam, float sg, float isg,
                                                      float tau, Dims d, int zc, const StopCtl* ctl,
                                                      double2* partials) {
    __shared__ float sU[2][BY * BX];
    __shared__ float sFx[2][BY * BX];
    __shared__ float sFy[2][BY * BX];
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 1;
    const int y = blockIdx.y * OY + ty - 1;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool o_pt = in_xy && tx >= 1 && tx <= BX - 2 && ty >= 1 && ty <= BY - 2;
    // upper neighbour in the tile, mirrored at the volume's upper edge (an axis
    // of length 1 maps to itself, Diffusion_core.c:255-265); lower neighbour
    // for the face flux shared with it
    int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    xh = min(max(xh, 0), BX - 1);
    yh = min(max(yh, 0), BY - 1);
    const int oc = ty * BX + tx;
    const int oxh = ty * BX + xh, oyh = yh * BX + tx;
    const int oxl = ty * BX + max(tx - 1, 0), oyl = max(ty - 1, 0) * BX + tx;
    const bool xlo = (x == 0), ylo = (y == 0);  // west / south mirror: w = U[i+1]
    const int col = min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    float pa = 0.f, pb = 0.f;

    if constexpr (!THREE) {
        const float u = __ldg(U + col);
        const float fv = o_pt ? __ldg(F + col) : 0.f;
        sU[0][oc] = u;
        __syncthreads();
        const float fxo = flux<PEN>(sU[0][oxh] - u, sg, isg);
        const float fyo = flux<PEN>(sU[0][oyh] - u, sg, isg);
        sFx[0][oc] = fxo;
        sFy[0][oc] = fyo;
        __syncthreads();
        if (o_pt) {
            const float w1 = xlo ? fxo : -sFx[0][oxl];
            const float s1 = ylo ? fyo : -sFy[0][oyl];
            const float sum = fxo + w1 + fyo + s1;
            const float un = u + tau * (lam * sum - (u - fv));
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
        const int sxy = (int)d.sxy;
        auto at = [&](int k) -> int { return min(max(k, 0), nz - 1) * sxy + col; };
        // registers entering step j: U(j-2), U(j-1), U(j), U(j+1); f of planes
        // j-2, j-1; own face fluxes of plane j-2 and the k flux of plane j-3
        float ua = __ldg(U + at(z0 - 2)), ub = __ldg(U + at(z0 - 1));
        float uc = __ldg(U + at(z0)), ud = __ldg(U + at(z0 + 1));
        float fa = 0.f, fb = 0.f;
        float fxo = 0.f, fyo = 0.f, fzo = 0.f, fzoo = 0.f;
        sU[1][oc] = ub;  // ring slot of plane p: (p - z0) & 1
        __syncthreads();

        auto step = [&](auto par, auto full, int j) {
            constexpr int P = decltype(par)::value;
            constexpr bool FULL = decltype(full)::value;
            const float ue = __ldg(U + at(j + 2));
            const float fe = o_pt ? __ldg(F + at(j)) : 0.f;
            // A. fluxes of plane m = j-1 through its upper faces
            const int m = j - 1;
            const float zhi = (m == nz - 1) ? ua : uc;  // mirrored k+1 (Diffusion_core.c:250)
            const float fx = flux<PEN>(sU[1 - P][oxh] - ub, sg, isg);
            const float fy = flux<PEN>(sU[1 - P][oyh] - ub, sg, isg);
            const float fz = flux<PEN>(zhi - ub, sg, isg);
            sFx[1 - P][oc] = fx;
            sFy[1 - P][oc] = fy;
            // B. publish U(j)
            sU[P][oc] = uc;
            // C. update plane j-2 (e, w, n, s, u, d as Diffusion_core.c:267-281)
            if (FULL) {
                const int kf = j - 2;
                const float w1 = xlo ? fxo : -sFx[P][oxl];
                const float s1 = ylo ? fyo : -sFy[P][oyl];
                const float d1 = (kf == 0) ? fzo : -fzoo;
                const float sum = fxo + w1 + fyo + s1 + fzo + d1;
                const float un = ua + tau * (lam * sum - (ua - fa));
                if (o_pt) Un[kf * sxy + col] = un;
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
            fb = fe;
            fzoo = fzo;
            fxo = fx;
            fyo = fy;
            fzo = fz;
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

template <bool THREE, bool CHECK>
cudaError_t launch(int pen, const NdfPlan& T, cudaStream_t s, const float* cur, float* nxt, const float* f,
                   float lam, float sg, float isg, float tau, const Dims& d, const StopCtl* ctl, double2* part) {
#define NDF_STREAM_CASE(P) \
    case P:                \
        return launch_pdl(k_ndf_stream<THREE, P, CHECK>, T.grid, T.block, 0, s, cur, nxt, f, lam, sg, isg, tau, d, \
                          T.zchunk, ctl, part);
    switch (pen) {
        NDF_STREAM_CASE(0)
        NDF_STREAM_CASE(1)
        NDF_STREAM_CASE(2)
        NDF_STREAM_CASE(3)
        NDF_STREAM_CASE(4)
        NDF_STREAM_CASE(5)
        default: break;
    }
#undef NDF_STREAM_CASE
    return cudaSuccess;
}

}  // namespace

NdfPlan ndf_stream_plan(const Dims& d) {
    if (ndf_pair_applies(d)) return ndf_pair_plan(d);
    NdfPlan T;
    const char* e = getenv("CILREG_NDF_KERNEL");
    // "simple" selects the per-voxel kernel; volumes of 2^31 voxels or more use
    // it too (the streaming kernel indexes with 32-bit offsets)
    T.use = !(e && strcmp(e, "simple") == 0) && d.n < (1LL << 31);
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_ndf_stream<true, 1, false>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 2, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int ndf_stream_step(const NdfPlan& T, int pen, const float* cur, float* nxt, const float* f, float lam, float sg,
                    float isg, float tau, const Dims& d, const StopCtl* ctl, int check, double2* partials,
                    cudaStream_t s) {
    if (T.pair) return ndf_pair_step(T, pen, cur, nxt, f, lam, sg, isg, tau, d, ctl, check, partials, s);
    if (d.nz > 1) {
        if (check)
            CILREG_CUDA((launch<true, true>(pen, T, s, cur, nxt, f, lam, sg, isg, tau, d, ctl, partials)));
        else
            CILREG_CUDA((launch<true, false>(pen, T, s, cur, nxt, f, lam, sg, isg, tau, d, ctl, partials)));
    } else {
        if (check)
            CILREG_CUDA((launch<false, true>(pen, T, s, cur, nxt, f, lam, sg, isg, tau, d, ctl, partials)));
        else
            CILREG_CUDA((launch<false, false>(pen, T, s, cur, nxt, f, lam, sg, isg, tau, d, ctl, partials)));
    }
    return OK;
}

}  // namespace cilreg
