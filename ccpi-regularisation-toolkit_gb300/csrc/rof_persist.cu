// ROF-TV on a 2D image at a fixed iteration count, all iterations in one
// persistent launch (reference arithmetic ROF_TV_core.c:102-160, 269-297).
//
// A 512^2 image takes about 2.4 us per iteration as one launch per iteration
// replayed from a CUDA graph, mostly the latency of a launch and of its
// single wave of CTAs, not its work.  Here each CTA keeps one 32 x 64 tile
// of U in shared memory for the whole run and exchanges only the tile's
// border with its eight neighbours through global memory (L2):
//   1. wait until the neighbour tiles have published iteration t (a flag per
//      tile, acquire loads, a bounded wait);
//   2. load the one-pixel halo ring of U^t from the global ping-pong buffer;
//   3. form the fluxes D1, D2 of the tile, of the row above it (D1) and of the
//      column left of it (D2), all with the reference's mirrored neighbours;
//   4. update the tile in place, write its border (the whole tile at the last
//      iteration) to the other global buffer, and release the tile's flag.
// Only neighbours synchronise: no grid-wide barrier.  A tile runs at most one
// iteration ahead of its neighbours (its next wait needs theirs), so a tile
// never overwrites a border that a neighbour has still to read.  Every tile
// must be resident at once: the launch is cooperative, and a wait that runs
// out sets an error word and the kernel leaves (the host then fails the call).
//
// Measured on a 512^2 image, 2000 iterations: 7.4-7.9 ms (3.7-3.9 us per
// iteration) against 4.75 ms for graph-replayed launches of k_rof_pair2d.  The
// chain release -> neighbour's acquire -> halo load through L2 costs more
// than a launch with programmatic dependent launch; dropping the fence before
// the release (9.4 ms) or the sleep in the poll (7.6 ms) did not help.  The
// kernel is therefore opt-in (CILREG_ROF_PERSIST=1).
//
// The arithmetic per pixel is that of k_rof_stream's 2D path, so the result
// equals one launch of that kernel per iteration bit for bit.  Data written
// within the launch is read through L2 (ld.global.cg).
#include <stdlib.h>

#include "rof_tiled.cuh"

namespace cilreg {

namespace {

constexpr int PW = 32, PH = 64;          // tile
constexpr int TX = 32, TY = 16;          // threads; each holds rows ty + 16 k, k = 0..3
constexpr int NTH = TX * TY;
constexpr int RS = PW + 2;               // shared row stride: columns -1 .. 32
constexpr int SROWS = PH + 2;            // rows -1 .. 64
constexpr int NHALO = 2 * (PW + 2) + 2 * PH;  // the halo ring: 196 points
constexpr long long WAIT_LIMIT = 1LL << 21;   // polls of a neighbour flag (about a second)

__device__ __forceinline__ int sidx(int c, int r) { return (r + 1) * RS + (c + 1); }

__device__ __forceinline__ float minmod_sq(float a, float b) {
    const float m = fmaxf(fminf(a, b), fminf(fmaxf(a, b), 0.f));
    return m * m;
}

struct PersistArgs {
    float* g0;  // U^t ping-pong: g0 holds U^0
    float* g1;
    const float* f;
    const float* lam_arr;  // per-pixel lambda or null
    float lam, tau;
    int iters;
    int* flags;  // one per tile, zero at launch
    int* error;  // set when a wait runs out
};

template <bool LARR>
__global__ void __launch_bounds__(NTH, 1) k_rof_persist2d(PersistArgs a, Dims d) {
    __shared__ float sU[SROWS * RS];
    __shared__ float sD1[SROWS * RS];
    __shared__ float sD2[SROWS * RS];
    __shared__ int s_abort;
    const float EPS = 1.0e-8f;
    const int nx = d.nx, ny = d.ny;
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
    const int gx = gridDim.x, gy = gridDim.y;
    const int bx = blockIdx.x, by = blockIdx.y, tile = by * gx + bx;
    const int x0 = bx * PW, y0 = by * PH;
    // mirrored neighbour offsets in shared memory of a point (c, r) at image
    // position (x, y) (ROF_TV_core.c:113-116; an axis of length 1 maps to itself)
    auto offs = [&](int c, int r, int x, int y, int& o, int& xl, int& xh, int& yl, int& yh) {
        o = sidx(c, r);
        xl = (nx == 1) ? o : ((x == 0) ? o + 1 : o - 1);
        xh = (nx == 1) ? o : ((x == nx - 1) ? o - 1 : o + 1);
        yl = (ny == 1) ? o : ((y == 0) ? o + RS : o - RS);
        yh = (ny == 1) ? o : ((y == ny - 1) ? o - RS : o + RS);
    };
    auto flux = [&](int o, int xl, int xh, int yl, int yh, float& d1, float& d2) {
        const float u = sU[o];
        const float xp = sU[xh] - u, xm = u - sU[xl];
        const float yp = sU[yh] - u, ym = u - sU[yl];
        const float mx2 = minmod_sq(xp, xm), my2 = minmod_sq(yp, ym);
        d1 = yp * rsqrtf(yp * yp + mx2 + EPS);
        d2 = xp * rsqrtf(xp * xp + my2 + EPS);
    };
    // D1 alone (row -1: needs no row -2) and D2 alone (column -1: needs no
    // column -2), with the same expressions
    auto flux_d1 = [&](int o, int xl, int xh, int yh) {
        const float u = sU[o];
        const float xp = sU[xh] - u, xm = u - sU[xl];
        const float yp = sU[yh] - u;
        const float mx2 = minmod_sq(xp, xm);
        return yp * rsqrtf(yp * yp + mx2 + EPS);
    };
    auto flux_d2 = [&](int o, int xh, int yl, int yh) {
        const float u = sU[o];
        const float xp = sU[xh] - u;
        const float yp = sU[yh] - u, ym = u - sU[yl];
        const float my2 = minmod_sq(yp, ym);
        return xp * rsqrtf(xp * xp + my2 + EPS);
    };
    // this thread's pixels: column tx, rows ty + 16 k
    const int x = x0 + tx;
    float fv[4], lv[4];
    int o[4], oxl[4], oxh[4], oyl[4], oyh[4];
    bool in[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int r = ty + TY * k, y = y0 + r;
        in[k] = x < nx && y < ny;
        const int g = min(y, ny - 1) * nx + min(x, nx - 1);
        offs(tx, r, x, y, o[k], oxl[k], oxh[k], oyl[k], oyh[k]);
        fv[k] = __ldg(a.f + g);
        lv[k] = LARR ? __ldg(a.lam_arr + g) : a.lam;
        sU[o[k]] = __ldg(a.g0 + g);
    }
    // the halo point this thread loads (tid < NHALO): row -1, row 64, column
    // -1, column 32; clamped into the image (outside it a halo point is never
    // read: the mirrors point inside the tile)
    int hs = 0, hg = 0;
    if (tid < NHALO) {
        int c, r;
        if (tid < PW + 2) {
            c = tid - 1, r = -1;
        } else if (tid < 2 * (PW + 2)) {
            c = tid - (PW + 2) - 1, r = PH;
        } else if (tid < 2 * (PW + 2) + PH) {
            c = -1, r = tid - 2 * (PW + 2);
        } else {
            c = PW, r = tid - 2 * (PW + 2) - PH;
        }
        hs = sidx(c, r);
        hg = min(max(y0 + r, 0), ny - 1) * nx + min(max(x0 + c, 0), nx - 1);
    }
    // the extra fluxes: warp 0 forms D2 of column -1 (rows lane, lane + 32),
    // warp 1 D1 of row -1 (column lane), at their mirrored neighbours; only
    // where a neighbour tile lies there (at the image edge the mirrors read
    // the tile's own fluxes instead)
    int eo[2] = {0, 0}, exl[2] = {0, 0}, exh[2] = {0, 0}, eyl[2] = {0, 0}, eyh[2] = {0, 0};
    const bool ex_col = ty == 0 && x0 > 0, ex_row = ty == 1 && y0 > 0;
    if (ex_col) {
#pragma unroll
        for (int k = 0; k < 2; k++) {
            const int r = tx + 32 * k;
            offs(-1, r, x0 - 1, min(y0 + r, ny - 1), eo[k], exl[k], exh[k], eyl[k], eyh[k]);
        }
    } else if (ex_row) {
        offs(tx, -1, min(x, nx - 1), y0 - 1, eo[0], exl[0], exh[0], eyl[0], eyh[0]);
    }
    // the neighbour tile this thread waits for: tid 0..7 take the 3 x 3
    // neighbourhood without its centre
    int nb = -1;
    if (tid < 8) {
        const int q = (tid < 4) ? tid : tid + 1;
        const int nbx = bx + (q % 3) - 1, nby = by + (q / 3) - 1;
        if (nbx >= 0 && nbx < gx && nby >= 0 && nby < gy) nb = nby * gx + nbx;
    }
    if (tid == 0) s_abort = 0;
    __syncthreads();

    const float tau = a.tau;
    for (int t = 0; t < a.iters; t++) {
        const float* G = (t & 1) ? a.g1 : a.g0;
        float* Gn = (t & 1) ? a.g0 : a.g1;
        // 1. the neighbours have published U^t
        if (t > 0 && nb >= 0) {
            long long polls = 0;
            while (ld_acquire_gpu(a.flags + nb) < t) {
                if (++polls > WAIT_LIMIT || ld_acquire_gpu(a.error) != 0) {
                    atomicExch(a.error, 1);
                    s_abort = 1;
                    break;
                }
                __nanosleep(32);
            }
        }
        __syncthreads();
        if (s_abort) break;
        // 2. the halo ring of U^t
        if (tid < NHALO) sU[hs] = __ldcg(G + hg);
        __syncthreads();
        // 3. fluxes (ROF_TV_core.c:102-160)
#pragma unroll
        for (int k = 0; k < 4; k++) flux(o[k], oxl[k], oxh[k], oyl[k], oyh[k], sD1[o[k]], sD2[o[k]]);
        if (ex_col) {
#pragma unroll
            for (int k = 0; k < 2; k++) sD2[eo[k]] = flux_d2(eo[k], exh[k], eyl[k], eyh[k]);
        } else if (ex_row) {
            sD1[eo[0]] = flux_d1(eo[0], exl[0], exh[0], eyh[0]);
        }
        __syncthreads();
        // 4. update in place (ROF_TV_core.c:269-297), publish the border
        const bool last = t == a.iters - 1;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float u = sU[o[k]];
            const float div = (sD1[o[k]] - sD1[oyl[k]]) + (sD2[o[k]] - sD2[oxl[k]]);
            const float un = u + tau * (lv[k] * div - (u - fv[k]));
            sU[o[k]] = un;
            const int r = ty + TY * k;
            const bool border = tx == 0 || tx == PW - 1 || r == 0 || r == PH - 1;
            if (in[k] && (border || last)) Gn[(y0 + r) * nx + x] = un;
        }
        __syncthreads();  // the border of U^{t+1} is written
        if (tid == 0) {
            __threadfence();
            st_release_gpu(a.flags + tile, t + 1);
        }
    }
}

}  // namespace

bool rof_persist2d_applies(const Dims& d, int iters) {
    // opt-in: CILREG_ROF_PERSIST=1 (and no kernel chosen by CILREG_ROF_KERNEL)
    const char* e = getenv("CILREG_ROF_PERSIST");
    const char* ek = getenv("CILREG_ROF_KERNEL");
    if (!(e && e[0] == '1') || (ek && ek[0] != '\0')) return false;
    if (d.nz != 1 || iters < 2 || d.n >= (1LL << 31)) return false;
    const long long tiles = (long long)((d.nx + PW - 1) / PW) * ((d.ny + PH - 1) / PH);
    int resident = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&resident, k_rof_persist2d<false>, NTH, 0) != cudaSuccess)
        resident = 0;
    cudaGetLastError();
    return tiles <= (long long)resident * sm_count();
}

long long rof_persist2d_tiles(const Dims& d) { return (long long)((d.nx + PW - 1) / PW) * ((d.ny + PH - 1) / PH); }

int rof_persist2d_run(float* g0, float* g1, const float* f, const float* lam_arr, float lam, float tau, int iters,
                      const Dims& d, int* flags, int* error, cudaStream_t s) {
    const dim3 grid((d.nx + PW - 1) / PW, (d.ny + PH - 1) / PH, 1), block(TX, TY, 1);
    CILREG_CUDA(cudaMemsetAsync(flags, 0, sizeof(int) * grid.x * grid.y, s));
    CILREG_CUDA(cudaMemsetAsync(error, 0, sizeof(int), s));
    PersistArgs a;
    a.g0 = g0;
    a.g1 = g1;
    a.f = f;
    a.lam_arr = lam_arr;
    a.lam = lam;
    a.tau = tau;
    a.iters = iters;
    a.flags = flags;
    a.error = error;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1] = {};
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (lam_arr)
        CILREG_CUDA(cudaLaunchKernelEx(&cfg, k_rof_persist2d<true>, a, d));
    else
        CILREG_CUDA(cudaLaunchKernelEx(&cfg, k_rof_persist2d<false>, a, d));
    return OK;
}

}  // namespace cilreg
