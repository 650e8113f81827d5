// FGP-TV iteration with the input planes staged by the Tensor Memory
// Accelerator (3D volumes whose x extent is a multiple of 4).
//
// Same tile, pipeline and arithmetic as k_fgp_stream (fgp_tiled.cu): a CTA
// of 32 x 16 threads on an overlapping x/y tile writes the inner 30 x 14
// voxels while walking a z chunk, two barriers per plane.  The seven input
// arrays of a plane (P^{k-1} and P^{k-2}, three components each, and f) are
// not loaded by the threads: one thread issues seven tensor copies
// (cp.async.bulk.tensor) of the tile's box per plane into a ring of STAGES
// shared-memory stages, STAGES - 1 planes ahead, completing on one mbarrier
// per stage; every thread then reads its own voxel's values from the stage.
// A stopping-check iteration also reads U_prev at each thread's own voxel,
// by plain loads one plane ahead (staging it as an eighth array would leave
// only three CTAs per SM).
// The box is 36 x 16 voxels starting at the tile's first x rounded down to a
// multiple of 4 (a tensor copy's x origin must be 16-byte aligned), and the
// thread reads column tx + r; voxels outside the volume (also planes below 0
// or past the end) arrive as zeros, which is the zero boundary the
// iteration needs.  Waits on an mbarrier are bounded: one that runs out sets
// an error flag that the host turns into a failed call.
#include <stdint.h>
#include <stdlib.h>

#include "fgp_tiled.cuh"
#include "tma_ring.cuh"

namespace cilreg {

namespace {

using namespace tma;

constexpr int BX = 32, BY = 16;          // threads
constexpr int OX = BX - 2, OY = BY - 2;  // output voxels per tile
constexpr int NT = BX * BY;
constexpr int BOX = BOXX * BY;           // floats per array per stage
constexpr int NIN = 7;                   // pc (3), po (3), f
// arrays staged (7, or 8 on check iterations) and ring depth (planes in
// flight + 1) per variant
template <bool CHECK, int ST>
struct Ring {
    static constexpr int NA = 7;  // U_prev (check iterations) is loaded by the threads
    static constexpr int STAGES = ST;
    static constexpr size_t DYN = sizeof(float) * BOX * NA * STAGES + 128;  // + alignment slack
};

__device__ int g_tma_timeout = 0;

struct TmaArgs {
    float* pn[3];
    float* u;
    float lam, c, multip;
    int nonneg, aniso, write_u, write_p;
};

struct TmaMaps {
    CUtensorMap m[NIN];  // pc[0..2], po[0..2], f
};

template <bool CHECK, int ST>
__global__ void __launch_bounds__(NT, CHECK ? 4 : 3) k_fgp_tma(const __grid_constant__ TmaMaps maps, TmaArgs a, Dims d, int zc,
                                                   const StopCtl* ctl, double2* partials) {
    extern __shared__ unsigned char dyn[];
    __shared__ float sR1[BY][BX];
    __shared__ float sR2[BY][BX];
    __shared__ float sU[2][BY][BX];
    constexpr int STAGES = Ring<CHECK, ST>::STAGES;
    constexpr int NA = Ring<CHECK, ST>::NA;
    __shared__ uint64_t bar[STAGES];
    if (ctl->stop) return;
    float* stage0 = (float*)(((uintptr_t)dyn + 127) & ~(uintptr_t)127);
    const int tx = threadIdx.x, ty = threadIdx.y;
    const bool leader = (tx == 0 && ty == 0);
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int xf = blockIdx.x * OX - 1;  // x of thread tx = 0
    const int yf = blockIdx.y * OY - 1;
    const int bx0 = box_x0(xf);
    const int rx = xf - bx0;
    const int x = xf + tx, y = yf + ty;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool u_pt = in_xy && tx >= 1 && ty >= 1;
    const bool p_pt = u_pt && tx <= OX && ty <= OY;
    const int col = in_xy ? (y * nx + x) : 0;
    const int sxy = (int)d.sxy;
    const int own = ty * BOXX + tx + rx;  // this thread's element in a stage array
    const int nplanes = z1 - z0 + 2;      // planes z0-1 .. z1
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
        for (int q = 0; q < NA; q++) load_box(dst + q * BOX, &maps.m[q], bx0, yf, z0 - 1 + p, &bar[s]);
    };
    if (leader)
        for (int p = 0; p < STAGES - 1 && p < nplanes; p++) issue(p);

    bool dead = false;
    float r1p = 0.f, r2p = 0.f, r3p = 0.f, up = 0.f;
    float uo = 0.f;
    float pa = 0.f, pb = 0.f;
    for (int k = z0 - 1; k <= z1; ++k) {
        const int p = k - (z0 - 1);
        // wait for plane k's stage (bounded), read this voxel's inputs
        if (!dead && !wait_stage(&bar[p % STAGES], p / STAGES)) {
            atomicExch(&g_tma_timeout, 1);
            dead = true;
        }
        const float* st = stage0 + (size_t)(p % STAGES) * BOX * NA + own;
        const float c1 = st[0 * BOX], c2 = st[1 * BOX], c3 = st[2 * BOX];
        const float o1 = st[3 * BOX], o2 = st[4 * BOX], o3 = st[5 * BOX];
        const float fk = st[6 * BOX];
        // 1. R of plane k
        const float r1 = c1 + a.c * (c1 - o1);
        const float r2 = c2 + a.c * (c2 - o2);
        const float r3 = c3 + a.c * (c3 - o3);
        // U_prev of plane k (check iterations; the voxel's own value, written by
        // the previous iteration), loaded one plane before it is consumed: a
        // plain load, not a staged box, so that the check variant needs the
        // plain one's shared memory and four CTAs still fit on an SM
        const float uo_next = (CHECK && p_pt && k >= z0 && k < z1) ? a.u[k * sxy + col] : 0.f;
        sR1[ty][tx] = r1;
        sR2[ty][tx] = r2;
        __syncthreads();
        // every thread has read plane k-1's stage: refill it with plane k+STAGES-1
        if (leader && p + STAGES - 1 < nplanes) {
            proxy_fence();
            issue(p + STAGES - 1);
        }
        // 2. U of plane k
        float u = 0.f;
        if (u_pt && k >= z0 && k < nz) {
            const float s = r1 + r2 + r3 - sR1[ty][tx - 1] - sR2[ty - 1][tx] - r3p;
            u = fk - a.lam * s;
            if (a.nonneg && u < 0.f) u = 0.f;
        }
        sU[k & 1][ty][tx] = u;
        __syncthreads();
        // 3. P^k of plane k-1
        const int kp = k - 1;
        if (p_pt && kp >= z0) {
            const int v = kp * sxy + col;
            if (CHECK) {
                const float df = up - uo;
                pa += df * df;
                pb += up * up;
            }
            if (a.write_u) a.u[v] = up;
            if (a.write_p) {
                const int ps = kp & 1;
                const float g1 = (x == nx - 1) ? 0.f : up - sU[ps][ty][tx + 1];
                const float g2 = (y == ny - 1) ? 0.f : up - sU[ps][ty + 1][tx];
                const float g3 = (kp != nz - 1) ? up - u : 0.f;
                float p1 = r1p + a.multip * g1;
                float p2 = r2p + a.multip * g2;
                float p3 = r3p + a.multip * g3;
                if (!a.aniso) {
                    const float den = p1 * p1 + p2 * p2 + p3 * p3;
                    const float sq = (den > 1.f) ? rsqrtf(den) : 1.f;
                    p1 = p1 * sq;
                    p2 = p2 * sq;
                    p3 = p3 * sq;
                } else {
                    p1 = unit_clip(p1);
                    p2 = unit_clip(p2);
                    p3 = unit_clip(p3);
                }
                a.pn[0][v] = p1;
                a.pn[1][v] = p2;
                a.pn[2][v] = p3;
            }
        }
        r1p = r1;
        r2p = r2;
        r3p = r3;
        up = u;
        uo = uo_next;
    }
    if (CHECK) block_pair_partial<NT>(pa, pb, partials, block_slot());
}

}  // namespace

bool fgp_tma_usable(const Dims& d) {
    const char* e = getenv("CILREG_FGP_TMA");
    if (e && e[0] == '0') return false;
    // row stride (nx floats) must be a multiple of 16 bytes; 32-bit offsets
    // below about 32 M voxels (256^3: 2.25 waves of CTAs) the thread-loading
    // kernel is as fast or faster; the staging pays off on large volumes
    const long long min_n = (e && e[0] == '1') ? 0 : (1LL << 25);
    return tma::volume_ok(d) && d.n >= min_n && d.n < (1LL << 31);
}

bool fgp_tma_encode(const float* const arrays[7], const Dims& d, void* maps_out) {
    TmaMaps* M = (TmaMaps*)maps_out;
    for (int q = 0; q < NIN; q++)
        if (!tma::encode(&M->m[q], arrays[q], d, BY)) return false;
    return true;
}

size_t fgp_tma_maps_bytes() { return sizeof(TmaMaps); }

namespace {

template <bool CHECK, int ST>
bool raise_smem_limit() {
    static const bool ok = [] {
        const bool r = cudaFuncSetAttribute(k_fgp_tma<CHECK, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)Ring<CHECK, ST>::DYN) == cudaSuccess;
        cudaGetLastError();
        return r;
    }();
    return ok;
}

template <bool CHECK, int ST>
int launch_tma(const TiledPlan& T, const TmaMaps& M, const TmaArgs& a, const Dims& d, const StopCtl* ctl,
               double2* partials, cudaStream_t s) {
    if (!raise_smem_limit<CHECK, ST>()) return fail(ERR_CUDA, __FILE__, __LINE__, "cannot raise the shared-memory limit of k_fgp_tma");
    k_fgp_tma<CHECK, ST><<<T.grid, T.block, Ring<CHECK, ST>::DYN, s>>>(M, a, d, T.zchunk, ctl, partials);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

// ring depth of the plain iterations: CILREG_FGP_TMA_STAGES (2..4, default 3)
int tma_stages() {
    static const int st = [] {
        const char* e = getenv("CILREG_FGP_TMA_STAGES");
        const int v = e ? atoi(e) : 3;
        return (v >= 2 && v <= 4) ? v : 3;
    }();
    return st;
}

}  // namespace

int fgp_tma_resident() {
    static const int r = [] {
        int n = 0;
        if (!raise_smem_limit<false, 3>() ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_fgp_tma<false, 3>, NT, Ring<false, 3>::DYN) !=
                cudaSuccess ||
            n <= 0)
            n = 3;
        cudaGetLastError();
        return n;
    }();
    return r;
}

int fgp_tma_step(const TiledPlan& T, const void* maps, float* const pn[3], float* u, float lam, float c,
                 float multip, int nonneg, int aniso, int write_u, int write_p, int check, const Dims& d,
                 const StopCtl* ctl, double2* partials, cudaStream_t s) {
    TmaArgs a;
    for (int i = 0; i < 3; i++) a.pn[i] = pn[i];
    a.u = u;
    a.lam = lam;
    a.c = c;
    a.multip = multip;
    a.nonneg = nonneg;
    a.aniso = aniso;
    a.write_u = write_u;
    a.write_p = write_p;
    const TmaMaps& M = *(const TmaMaps*)maps;
    if (check) return launch_tma<true, 3>(T, M, a, d, ctl, partials, s);
    switch (tma_stages()) {
        case 2: return launch_tma<false, 2>(T, M, a, d, ctl, partials, s);
        case 4: return launch_tma<false, 4>(T, M, a, d, ctl, partials, s);
        default: return launch_tma<false, 3>(T, M, a, d, ctl, partials, s);
    }
}

int fgp_tma_status(cudaStream_t s) {
    int h = 0;
    CILREG_CUDA(cudaMemcpyFromSymbolAsync(&h, g_tma_timeout, sizeof(int), 0, cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (h) {
        const int zero = 0;
        CILREG_CUDA(cudaMemcpyToSymbolAsync(g_tma_timeout, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, s));
        CILREG_CUDA(cudaStreamSynchronize(s));
        return fail(ERR_CUDA, __FILE__, __LINE__, "a tensor-copy wait in k_fgp_tma timed out");
    }
    return OK;
}

}  // namespace cilreg
