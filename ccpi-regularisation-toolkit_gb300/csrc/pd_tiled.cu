// PD-TV iteration as a 2.5D streaming stencil (2D images are the nz == 1 case).
//
// Reference arithmetic: PD_TV_core.c:212-252 (dual ascent with mirrored
// forward differences, projection utils.c:180-213, nonnegativity after the
// dual step, primal step with the backward divergence, extrapolation).
// A CTA of 32 x 16 threads holds an overlapping tile: thread (tx, ty) sits on
// voxel (x0 - 1 + tx, y0 - 1 + ty); the projected dual P' is formed on
// tx <= 30, ty <= 14 and the primal update on the inner 30 x 14 voxels.
// Step j of each thread, walking a chunk of z planes:
//   A. forms P'(j-1) once per voxel from Ue of plane j-1 (x/y forward
//      neighbours from shared memory, z from its own registers, mirrored at
//      the last index) and the old dual, then projects it; the x and y
//      components go to shared memory for the backward divergence;
//   B. publishes Ue(j) (loaded one step earlier) to shared memory;
//   C. after one barrier, updates plane j-1: U = (clamp(Ue) - tau div P' +
//      lt f) / (1 + lt), writes Ue' = U + theta (U - clamp(Ue)) and P'.
// HBM traffic: read Ue, P(3), f; write Ue, P(3) -> 36 B per voxel (28 in 2D).
#include <stdlib.h>
#include <string.h>

#include "pd_tiled.cuh"
#include "pd_math.cuh"

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 2, OY = BY - 2;
constexpr int NT = BX * BY;
constexpr int ZCHUNK = 64;

// CHECK: a stopping-check iteration (writes U before extrapolation and the
// per-CTA partial sums).  IT: element-offset type (int below 2^31 voxels).
template <bool THREE, bool CHECK, typename IT>
__global__ void __launch_bounds__(NT, 3) k_pd_stream(PdStreamArgs a, Dims d, int zc, const StopCtl* ctl,
                                                     double2* partials) {
    __shared__ float sUe[2][BY][BX];
    __shared__ float sP1[2][BY][BX];
    __shared__ float sP2[2][BY][BX];
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 1;
    const int y = blockIdx.y * OY + ty - 1;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool p_pt = in_xy && tx <= BX - 2 && ty <= BY - 2;   // dual formed here
    const bool o_pt = in_xy && tx >= 1 && ty >= 1 && tx <= OX && ty <= OY;  // update written here
    // mirrored forward neighbour inside the tile (length-1 axis -> itself)
    const int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    const int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    const IT col = in_xy ? ((IT)y * nx + x) : 0;
    const IT sxy = (IT)d.sxy;

    auto ld = [&](const float* p, int k) -> float {
        return (in_xy && k >= 0 && k < nz) ? __ldg(p + ((IT)k * sxy + col)) : 0.f;
    };
    // registers: Ue of planes j-2, j-1, j; prefetched Ue(j+1), old dual and f of plane j
    float um2 = ld(a.u, z0 - 2), um1 = ld(a.u, z0 - 1), uj = ld(a.u, z0);
    float q1 = ld(a.p[0], z0 - 1), q2 = ld(a.p[1], z0 - 1), q3 = THREE ? ld(a.p[2], z0 - 1) : 0.f;
    float fq = ld(a.f, z0 - 1);
    float p3m = 0.f;  // projected z component of the previous plane
    float pa = 0.f, pb = 0.f;
    sUe[(z0 - 1) & 1][ty][tx] = um1;
    __syncthreads();

    for (int j = z0; j <= z1; ++j) {
        const int k = j - 1;  // plane of this step's dual and update
        // prefetch for the next step: Ue(j+1), old dual and f of plane j
        const float un1 = (j + 1 <= z1) ? ld(a.u, j + 1) : 0.f;
        const float nq1 = ld(a.p[0], j), nq2 = ld(a.p[1], j), nq3 = THREE ? ld(a.p[2], j) : 0.f;
        const float nf = ld(a.f, j);
        // A. projected dual of plane k
        float p1 = 0.f, p2 = 0.f, p3 = 0.f;
        const bool plane_ok = (k >= 0) && (k >= z0 - 1) && (k < z1);
        if (plane_ok && p_pt) {
            const int sk = k & 1;
            const float c = sUe[sk][ty][tx];
            p1 = pd_dual(q1, a.sigma, sUe[sk][ty][xh], c);
            p2 = pd_dual(q2, a.sigma, sUe[sk][yh][tx], c);
            if (THREE) {
                const float zhi = (nz == 1) ? c : ((k + 1 >= nz) ? um2 : uj);  // mirrored (PD_TV_core.c:225)
                p3 = pd_dual(q3, a.sigma, zhi, c);
            }
            if (!a.aniso) {
                pd_project_iso<THREE>(p1, p2, p3);
            } else {
                p1 = pd_project_aniso(p1);
                p2 = pd_project_aniso(p2);
                p3 = pd_project_aniso(p3);
            }
            sP1[sk][ty][tx] = p1;
            sP2[sk][ty][tx] = p2;
        }
        // B. publish Ue(j)
        sUe[j & 1][ty][tx] = uj;
        __syncthreads();
        // C. primal update of plane k
        if (o_pt && k >= z0 && k < z1) {
            const int sk = k & 1;
            const float d1 = (x == 0) ? -p1 : -(p1 - sP1[sk][ty][tx - 1]);
            const float d2 = (y == 0) ? -p2 : -(p2 - sP2[sk][ty - 1][tx]);
            float dv = d1 + d2;
            if (THREE) {
                const float d3 = (k == 0) ? -p3 : -(p3 - p3m);
                dv = dv + d3;
            }
            float uc = um1;
            if (a.nonneg && uc < 0.f) uc = 0.f;
            const float unew = pd_primal(uc, a.tau, dv, a.lt, fq, a.onelt);
            const IT v = (IT)k * sxy + col;
            if (CHECK) {
                const float df = unew - uc;
                pa += df * df;
                pb += unew * unew;
                a.ubrk[v] = unew;
            }
            a.un[v] = pd_extrapolate(unew, a.theta, uc);
            a.pn[0][v] = p1;
            a.pn[1][v] = p2;
            if (THREE) a.pn[2][v] = p3;
        }
        p3m = p3;
        um2 = um1;
        um1 = uj;
        uj = un1;
        q1 = nq1;
        q2 = nq2;
        q3 = nq3;
        fq = nf;
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// One 2D iteration (nz == 1) on the tile of k_pd_stream without its plane
// pipeline: Ue, the dual and f of the image are loaded at once (f before the
// wait on the previous iteration), then the dual (one barrier) and the primal
// update (a second barrier), with k_pd_stream's expressions, so the iterates
// are the same bit for bit.
template <bool CHECK>
__global__ void __launch_bounds__(NT, 3) k_pd_2d(PdStreamArgs a, Dims d, int zc, const StopCtl* ctl,
                                                 double2* partials) {
    __shared__ float sUe[BY][BX];
    __shared__ float sP1[BY][BX];
    __shared__ float sP2[BY][BX];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int nx = d.nx, ny = d.ny;
    const int x = blockIdx.x * OX + tx - 1;
    const int y = blockIdx.y * OY + ty - 1;
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool p_pt = in_xy && tx <= BX - 2 && ty <= BY - 2;
    const bool o_pt = in_xy && tx >= 1 && ty >= 1 && tx <= OX && ty <= OY;
    const int xh = (nx == 1) ? tx : ((x + 1 >= nx) ? tx - 1 : tx + 1);
    const int yh = (ny == 1) ? ty : ((y + 1 >= ny) ? ty - 1 : ty + 1);
    const int col = in_xy ? (y * nx + x) : 0;
    const float fq = in_xy ? __ldg(a.f + col) : 0.f;  // f never changes: loaded before the wait
    pdl_wait();  // the previous iteration has completed (launch_pdl)
    pdl_trigger();
    if (ctl->stop) return;
    float c = 0.f, q1 = 0.f, q2 = 0.f;
    if (in_xy) {
        c = __ldg(a.u + col);
        q1 = __ldg(a.p[0] + col);
        q2 = __ldg(a.p[1] + col);
    }
    sUe[ty][tx] = c;
    __syncthreads();
    float p1 = 0.f, p2 = 0.f, p3 = 0.f;
    if (p_pt) {
        p1 = pd_dual(q1, a.sigma, sUe[ty][xh], c);
        p2 = pd_dual(q2, a.sigma, sUe[yh][tx], c);
        if (!a.aniso) {
            pd_project_iso<false>(p1, p2, p3);
        } else {
            p1 = pd_project_aniso(p1);
            p2 = pd_project_aniso(p2);
        }
        sP1[ty][tx] = p1;
        sP2[ty][tx] = p2;
    }
    __syncthreads();
    float pa = 0.f, pb = 0.f;
    if (o_pt) {
        const float d1 = (x == 0) ? -p1 : -(p1 - sP1[ty][tx - 1]);
        const float d2 = (y == 0) ? -p2 : -(p2 - sP2[ty - 1][tx]);
        const float dv = d1 + d2;
        float uc = c;
        if (a.nonneg && uc < 0.f) uc = 0.f;
        const float unew = pd_primal(uc, a.tau, dv, a.lt, fq, a.onelt);
        if (CHECK) {
            const float df = unew - uc;
            pa = df * df;
            pb = unew * unew;
            a.ubrk[col] = unew;
        }
        a.un[col] = pd_extrapolate(unew, a.theta, uc);
        a.pn[0][col] = p1;
        a.pn[1][col] = p2;
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

}  // namespace

PdPlan pd_stream_plan(const Dims& d) {
    PdPlan T;
    T.block = dim3(BX, BY, 1);
    if (d.nz > 1) {
        static const int resident = resident_ctas(k_pd_stream<true, false, int>, NT);
        const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
        T.zchunk = wave_zchunk(tiles, d.nz, resident, 1, ZCHUNK);
    } else {
        T.zchunk = 1;
    }
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int pd_stream_step(const PdPlan& T, const PdStreamArgs& a, const Dims& d, const StopCtl* ctl, double2* partials,
                   cudaStream_t s) {
    const bool three = d.nz > 1, check = a.check != 0;
    decltype(&k_pd_stream<true, true, int>) kern;
    // 2D images below 2^31 pixels: the kernel without the plane pipeline
    // (CILREG_PD_KERNEL=stream keeps the streaming kernel)
    const char* ek = getenv("CILREG_PD_KERNEL");
    if (!three && d.n < (1LL << 31) && !(ek && strcmp(ek, "stream") == 0))
        kern = check ? k_pd_2d<true> : k_pd_2d<false>;
    else if (d.n < (1LL << 31))
        kern = three ? (check ? k_pd_stream<true, true, int> : k_pd_stream<true, false, int>)
                     : (check ? k_pd_stream<false, true, int> : k_pd_stream<false, false, int>);
    else
        kern = three ? (check ? k_pd_stream<true, true, long long> : k_pd_stream<true, false, long long>)
                     : (check ? k_pd_stream<false, true, long long> : k_pd_stream<false, false, long long>);
    CILREG_CUDA(launch_pdl(kern, T.grid, T.block, 0, s, a, d, T.zchunk, ctl, partials));
    return OK;
}

}  // namespace cilreg
