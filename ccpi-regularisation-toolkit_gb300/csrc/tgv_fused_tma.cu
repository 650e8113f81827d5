// The one-pass TGV iteration (tgv_fused.cu) with every input plane staged by
// the Tensor Memory Accelerator (3D volumes whose x extent is a multiple of 4).
//
// Same tile (32 x 16 threads, the dual formed on 31 x 15, the primal written
// on the inner 30 x 14), same z walk and the same per-voxel arithmetic
// (tgv_fused_math.cuh), so the iterates equal the thread-loading pass bit for
// bit.  What changes is how the 14 input arrays of a plane (U, V1..V3,
// P1..P3, Q1..Q6, U0) reach the threads: one thread issues 14 tensor copies
// (cp.async.bulk.tensor) of the tile's box into a ring of three shared-memory
// stages, completing on one mbarrier per stage, and every thread reads its
// voxel and its forward x / y neighbours from the stage.  The thread-loading
// pass fetches P, Q and U0 in the step that uses them and holds U, V two
// planes ahead in registers, so at two CTAs per SM (64 registers) the load
// latency is exposed; here a plane is requested about one and a half steps
// before its first use and the threads hold no load registers.
//
// Step p of a CTA (plane j = z0 - 1 + p) needs the stages of planes j (its
// own values and the x / y neighbours for the forward differences) and j + 1
// (the z neighbour).  Each thread reads everything it needs from stage j
// before the dual half's barrier, so once that barrier is passed the stage is
// free and the issuing thread refills it with plane j + 3.
//
// Boxes are 36 x 16 floats from the tile's first x rounded down to a multiple
// of 4 (a tensor copy's x origin must be 16-byte aligned); the thread reads
// column tx + r.  Voxels outside the volume (and planes before the first or
// after the last) arrive as zeros; no voxel outside the volume is used (the
// forward neighbour of a last voxel is never read, halo threads outside the
// volume form nothing).  Waits on an mbarrier are bounded: one that runs out
// sets an error flag that the host turns into a failed call.
#include <stdint.h>
#include <stdlib.h>

#include "tgv_fused_math.cuh"
#include "tgv_tiled.cuh"
#include "tma_ring.cuh"

namespace cilreg {

namespace {

using namespace tma;

constexpr int BX = 32, BY = 16;
constexpr int OX = BX - 2, OY = BY - 2;
constexpr int NT = BX * BY;
constexpr int BOX = BOXX * BY;  // floats per array per stage
constexpr int NA = 14;          // U, V1..V3, P1..P3, Q1..Q6, U0
constexpr int STAGES = 3;
constexpr int A_U = 0, A_V = 1, A_P = 4, A_Q = 7, A_U0 = 13;
constexpr size_t DYN = sizeof(float) * BOX * NA * STAGES + 128;  // + alignment slack

__device__ int g_tgv_tma_timeout = 0;

struct TgvMaps {
    CUtensorMap m[NA];
};

// One tile (bx, by, bz) of one volume.  maps: the volume's 14 tensor maps
// (a kernel parameter, or device memory in batched runs); A: the argument
// block, a kernel parameter or (batched runs) a volatile copy in shared
// memory, read at each use rather than held in registers.
template <bool CHECK, class A>
__device__ __forceinline__ void tma_tile(const CUtensorMap* maps, A& a, const Dims& d, int zc, int bx, int by,
                                         int bz, float& pa_out, float& pb_out) {
    extern __shared__ unsigned char dyn[];
    __shared__ float sPQ[7][BY * BX];  // new P1, P2, Q1, Q2, Q4, Q5, Q6 of plane j
    __shared__ uint64_t bar[STAGES];
    float* stage0 = (float*)(((uintptr_t)dyn + 127) & ~(uintptr_t)127);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const bool leader = (tx == 0 && ty == 0);
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int xf0 = bx * OX - 1;  // x of thread tx = 0
    const int yf0 = by * OY - 1;
    const int bx0 = box_x0(xf0);
    const int rx = xf0 - bx0;
    const int x = xf0 + tx, y = yf0 + ty;
    const int z0 = bz * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool d_pt = in_xy && tx <= BX - 2 && ty <= BY - 2;  // dual formed here
    const bool o_pt = d_pt && tx >= 1 && ty >= 1;               // primal formed and written here
    const bool xe = (x == nx - 1), ye = (y == ny - 1), xf = (x == 0), yf = (y == 0);
    const int oc = ty * BX + tx;
    const int oxl = ty * BX + max(tx - 1, 0), oyl = max(ty - 1, 0) * BX + tx;
    // this thread's element of a stage array and its forward x / y neighbours
    // (clamped into the box: a clamped neighbour is never used)
    const int own = ty * BOXX + tx + rx;
    const int sxh = ty * BOXX + min(tx + 1, BX - 1) + rx;
    const int syh = min(ty + 1, BY - 1) * BOXX + tx + rx;
    const int col = in_xy ? (y * nx + x) : 0;
    const int sxy = (int)d.sxy;
    const float sigma = a.sigma, tau = a.tau, lam = a.lambda, ilt = a.inv_lt;
    const float alpha1 = a.alpha1, alpha0 = a.alpha0;
    const int nplanes = z1 - z0 + 2;  // planes z0-1 .. z1
    constexpr uint32_t STAGE_BYTES = sizeof(float) * BOX * NA;

    if (leader) {
        for (int s = 0; s < STAGES; s++) mbar_init(&bar[s]);
        mbar_init_fence();
    }
    __syncthreads();
    auto issue = [&](int p) {  // plane z0-1+p into stage p % STAGES
        const int s = p % STAGES;
        float* dst = stage0 + (size_t)s * BOX * NA;
        mbar_expect(&bar[s], STAGE_BYTES);
        for (int q = 0; q < NA; q++) load_box(dst + q * BOX, maps + q, bx0, yf0, z0 - 1 + p, &bar[s]);
    };
    if (leader)
        for (int p = 0; p < STAGES && p < nplanes; p++) issue(p);

    bool dead = false;
    auto wait = [&](int p) {
        if (!dead && !wait_stage(&bar[p % STAGES], p / STAGES)) {
            atomicExch(&g_tgv_tma_timeout, 1);
            dead = true;
        }
    };
    wait(0);
    // new P3, Q3, Q5, Q6 of plane j-1 (z predecessors of the divergences)
    float zp3 = 0.f, zq3 = 0.f, zq5 = 0.f, zq6 = 0.f;
    float pa = 0.f, pb = 0.f;

    for (int p = 0; p + 1 < nplanes; ++p) {
        const int j = z0 - 1 + p;
        wait(p + 1);
        const float* sc = stage0 + (size_t)(p % STAGES) * BOX * NA;        // plane j
        const float* sn = stage0 + (size_t)((p + 1) % STAGES) * BOX * NA;  // plane j+1
        const bool plane_ok = (j >= 0);
        const int o = (plane_ok ? j : 0) * sxy + col;
        // the values the primal half needs after the stage is refilled
        const float cu = sc[A_U * BOX + own];
        const float v1 = sc[(A_V + 0) * BOX + own], v2 = sc[(A_V + 1) * BOX + own], v3 = sc[(A_V + 2) * BOX + own];
        const float u0 = sc[A_U0 * BOX + own];
        // dual half at plane j (DualP_3D + ProjP_3D, DualQ_3D + ProjQ_3D)
        TgvDual n{};
        if (d_pt && plane_ok) {
            float pq[9];
            for (int i = 0; i < 3; i++) pq[i] = sc[(A_P + i) * BOX + own];
            for (int i = 0; i < 6; i++) pq[3 + i] = sc[(A_Q + i) * BOX + own];
            n = tgv_dual_voxel(
                cu, v1, v2, v3, [&](int c) { return sc[(A_U + c) * BOX + sxh]; },
                [&](int c) { return sc[(A_U + c) * BOX + syh]; }, [&](int c) { return sn[(A_U + c) * BOX + own]; },
                pq, xe, ye, j == nz - 1, sigma, alpha1, alpha0);
            if (o_pt && j >= z0) {
                a.pn[0][o] = n.p1;
                a.pn[1][o] = n.p2;
                a.pn[2][o] = n.p3;
                a.qn[0][o] = n.q1;
                a.qn[1][o] = n.q2;
                a.qn[2][o] = n.q3;
                a.qn[3][o] = n.q4;
                a.qn[4][o] = n.q5;
                a.qn[5][o] = n.q6;
            }
        }
        __syncthreads();  // every thread has read the previous plane's sPQ
        sPQ[0][oc] = n.p1;
        sPQ[1][oc] = n.p2;
        sPQ[2][oc] = n.q1;
        sPQ[3][oc] = n.q2;
        sPQ[4][oc] = n.q4;
        sPQ[5][oc] = n.q5;
        sPQ[6][oc] = n.q6;
        __syncthreads();  // sPQ of plane j is complete, and no thread reads plane j's stage any more
        if (leader && p + STAGES < nplanes) {
            proxy_fence();
            issue(p + STAGES);
        }
        // primal half at plane j (DivProjP_3D + newU3D, UpdV_3D + newV)
        if (o_pt && j >= z0) {
            const bool zf = (j == 0), zl = (j == nz - 1);
            const float ue =
                tgv_primal_u(n, sPQ[0][oxl], sPQ[1][oyl], zp3, xf, xe, yf, ye, zf, zl, cu, u0, lam, tau, ilt);
            a.un[o] = ue;
            if (CHECK) {
                const float df = ue - cu;
                pa += df * df;
                pb += ue * ue;
            }
            const TgvNewV w = tgv_primal_v(n, sPQ[2][oxl], sPQ[4][oxl], sPQ[5][oxl], sPQ[3][oyl], sPQ[4][oyl],
                                           sPQ[6][oyl], zq3, zq5, zq6, xf, xe, yf, ye, zf, zl, v1, v2, v3, tau);
            a.vn[0][o] = w.v1;
            a.vn[1][o] = w.v2;
            a.vn[2][o] = w.v3;
        }
        zp3 = n.p3;
        zq3 = n.q3;
        zq5 = n.q5;
        zq6 = n.q6;
    }
    pa_out = pa;
    pb_out = pb;
}

template <bool CHECK>
__global__ void __launch_bounds__(NT, 2) k_tgv_fused_tma(const __grid_constant__ TgvMaps maps, TgvFusedArgs a,
                                                         Dims d, int zc, const StopCtl* ctl, double2* partials) {
    if (ctl->stop) return;
    float pa = 0.f, pb = 0.f;
    tma_tile<CHECK, TgvFusedArgs>(maps.m, a, d, zc, blockIdx.x, blockIdx.y, blockIdx.z, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

// one iteration of every volume of a batch: a flat grid over all volumes'
// tiles; `parity` selects the (old, new) buffer pair of the iteration and the
// tensor maps of its old buffers (maps + (2 v + parity) x 14 for volume v)
template <bool CHECK>
__global__ void __launch_bounds__(NT, 2) k_tgv_fused_tma_batch(const TgvFusedVol* __restrict__ vols,
                                                               const int* __restrict__ tile_vol,
                                                               const CUtensorMap* __restrict__ maps, int parity) {
    __shared__ TgvFusedArgs sa;
    const long long t = blockIdx.x;
    const int v = tile_vol[t];
    const TgvFusedVol& V = vols[v];
    if (V.ctl->stop) return;
    const long long lt = t - V.tile_base;
    const int bx = (int)(lt % V.gx);
    const int by = (int)((lt / V.gx) % V.gy);
    const int bz = (int)(lt / ((long long)V.gx * V.gy));
    if (threadIdx.x == 0 && threadIdx.y == 0) sa = V.args[parity];
    __syncthreads();
    volatile TgvFusedArgs& va = sa;
    float pa = 0.f, pb = 0.f;
    tma_tile<CHECK, volatile TgvFusedArgs>(maps + ((size_t)v * 2 + parity) * NA, va, V.d, V.zc, bx, by, bz, pa, pb);
    if (CHECK) block_pair_partial<NT>(pa, pb, V.partials, lt);
}

template <bool CHECK>
bool raise_smem_limit() {
    static const bool ok = [] {
        const bool r =
            cudaFuncSetAttribute(k_tgv_fused_tma<CHECK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DYN) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_tgv_fused_tma_batch<CHECK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)DYN) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    return ok;
}

}  // namespace

bool tgv_tma_usable(const Dims& d) {
    const char* e = getenv("CILREG_TGV_TMA");
    if (e && e[0] == '0') return false;
    return tma::volume_ok(d) && d.n < (1LL << 31) && tgv_tma_resident() >= 2;
}

int tgv_tma_resident() {
    static const int r = [] {
        int n = 0, nb = 0;
        if (!raise_smem_limit<false>() || !raise_smem_limit<true>() ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_tgv_fused_tma<false>, NT, DYN) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_tgv_fused_tma_batch<false>, NT, DYN) !=
                cudaSuccess)
            n = nb = 0;
        cudaGetLastError();
        return n < nb ? n : nb;
    }();
    return r;
}

bool tgv_tma_batch_usable(const Dims* dims, int nvol) {
    const char* e = getenv("CILREG_TGV_TMA");
    if (e && e[0] == '0') return false;
    for (int v = 0; v < nvol; v++)
        if (!tma::volume_ok(dims[v]) || dims[v].n >= (1LL << 31)) return false;
    return tgv_tma_resident() >= 2;
}

int tgv_tma_batch_step(const TgvFusedVol* d_vols, const int* d_tile_vol, const void* d_maps, long long ntiles,
                       int parity, int check, cudaStream_t s) {
    if (ntiles < 1 || ntiles > 2147483647LL) return fail(ERR_ARG, __FILE__, __LINE__, "tile count %lld", ntiles);
    if (!raise_smem_limit<false>() || !raise_smem_limit<true>())
        return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_tgv_fused_tma_batch");
    const CUtensorMap* maps = (const CUtensorMap*)d_maps;
    if (check)
        k_tgv_fused_tma_batch<true><<<dim3((unsigned)ntiles), dim3(BX, BY, 1), DYN, s>>>(d_vols, d_tile_vol, maps,
                                                                                         parity);
    else
        k_tgv_fused_tma_batch<false><<<dim3((unsigned)ntiles), dim3(BX, BY, 1), DYN, s>>>(d_vols, d_tile_vol, maps,
                                                                                          parity);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

size_t tgv_tma_maps_bytes() { return sizeof(TgvMaps); }

bool tgv_tma_encode(const TgvFusedArgs& a, const Dims& d, void* maps_out) {
    TgvMaps* M = (TgvMaps*)maps_out;
    const float* arrays[NA] = {a.u,    a.v[0], a.v[1], a.v[2], a.p[0], a.p[1], a.p[2],
                               a.q[0], a.q[1], a.q[2], a.q[3], a.q[4], a.q[5], a.u0};
    for (int q = 0; q < NA; q++)
        if (!tma::encode(&M->m[q], arrays[q], d, BY)) return false;
    return true;
}

int tgv_tma_step(const TgvPlan& T, const void* maps, const TgvFusedArgs& a, const Dims& d, const StopCtl* ctl,
                 int check, double2* partials, cudaStream_t s) {
    const TgvMaps& M = *(const TgvMaps*)maps;
    if (!raise_smem_limit<false>() || !raise_smem_limit<true>())
        return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_tgv_fused_tma");
    if (check)
        k_tgv_fused_tma<true><<<T.grid, T.block, DYN, s>>>(M, a, d, T.zchunk, ctl, partials);
    else
        k_tgv_fused_tma<false><<<T.grid, T.block, DYN, s>>>(M, a, d, T.zchunk, ctl, partials);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

int tgv_tma_status(cudaStream_t s) {
    int h = 0;
    CILREG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_tgv_tma_timeout, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (h) {
        const int zero = 0;
        CILREG_CUDA(cudaMemcpyToSymbolAsync(g_tgv_tma_timeout, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
        CILREG_CUDA(cudaStreamSynchronize(s));
        return fail(ERR_CUDA, __FILE__, __LINE__, "a tensor-copy wait in k_tgv_fused_tma timed out");
    }
    return OK;
}

}  // namespace cilreg
