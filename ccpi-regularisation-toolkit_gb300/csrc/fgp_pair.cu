// Two FGP-TV iterations in one 2.5D streaming pass (temporal blocking, 3D).
//
// Iterations k and k+1 read P^{k-1}, P^{k-2} and f once and write P^k and
// P^{k+1}: 52 B per voxel for two iterations instead of 80.  A CTA of
// 32 x 16 threads holds a tile with a two-voxel halo (thread (tx, ty) on
// voxel (x0 - 2 + tx, y0 - 2 + ty)) and writes the inner 28 x 12 voxels.
// Level 1 is the single-iteration pipeline of fgp_tiled.cu on the whole
// tile (R^k, U^k, then P^k one plane behind, valid on the inner 30 x 14);
// level 2 runs the same pipeline on level 1's P^k two planes behind it:
//   R^{k+1} = P^k + c_{k+1} (P^k - P^{k-1}),  U^{k+1} = f - lambda div_b R^{k+1},
//   P^{k+1} = proj(R^{k+1} + m grad_f U^{k+1}),
// so U^{k+1} is valid on the inner 29 x 13 and P^{k+1} on the inner 28 x 12.
// Step j of each thread, walking its z chunk:
//   A. level 1 forms R^k(j), level 2 forms R^{k+1}(j-2) from the P^k(j-2)
//      level 1 left in registers; both publish their x/y components;
//   B. (barrier) U^k(j) and U^{k+1}(j-2); both published;
//   C. (barrier) P^k(j-1) and P^{k+1}(j-3), each from the U plane published
//      one step earlier (x/y forward neighbours) and the U just formed (z).
// The inputs reach shared memory by asynchronous 4-byte copies issued AHEAD
// planes early into a ring of AHEAD + 3 planes; each thread reads only the
// elements it copied itself (its own voxel), so the copies need no barrier,
// and level 2 re-reads P^{k-1}(j-2) and f(j-2) from the ring.  Every
// arithmetic expression is the one of fgp_tiled.cu, so a pair gives the same
// P^k, P^{k+1} as two single iterations.  No stopping check runs inside a
// pair (checks run as single iterations).
//
// Measured at 256^3 (ncu): 315 us per pair against 121 us per single
// iteration, with 51.5 B per voxel of DRAM traffic per pair as designed; the
// pass is bound by instruction issue (2.4x the single kernel's instructions
// per step, at 62 registers two CTAs per SM instead of three) and by barrier
// stalls, not by DRAM.  Pairs are therefore opt-in (CILREG_FGP_PAIR=1).
#include "fgp_tiled.cuh"

#include <stdlib.h>

#include <type_traits>

namespace cilreg {

namespace {

constexpr int BX = 32, BY = 16;          // threads
constexpr int OX = BX - 4, OY = BY - 4;  // output voxels per tile
constexpr int NT = BX * BY;
constexpr int AHEAD = 3;
constexpr int RING = AHEAD + 3;  // planes j-2 .. j+AHEAD
constexpr int NIN = 7;           // pc (3), po (3), f
constexpr int ZCHUNK = 64;
constexpr size_t RING_BYTES = sizeof(float) * RING * NIN * NT;

template <int V>
using Ic = std::integral_constant<int, V>;

struct PairArgs {
    const float* pc[3];  // P^{k-1}
    const float* po[3];  // P^{k-2}
    float* pn1[3];       // P^k
    float* pn2[3];       // P^{k+1}
    const float* f;
    float* u;            // U^{k+1} when write_u2
    float lam, c1, c2, multip;
    int nonneg, aniso, write_u2, write_p2;
};

__device__ __forceinline__ void cp_async4_zfill(float* sdst, const float* gsrc, bool valid) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
    const int n = valid ? 4 : 0;  // 0: nothing is read, the element is zero-filled
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gsrc), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit_group() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// P update and projection of fgp_tiled.cu (same expressions)
__device__ __forceinline__ void p_update(float r1, float r2, float r3, float g1, float g2, float g3, float multip,
                                         int aniso, float& p1, float& p2, float& p3) {
    p1 = r1 + multip * g1;
    p2 = r2 + multip * g2;
    p3 = r3 + multip * g3;
    if (!aniso) {
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
}

template <typename IT>
__global__ void __launch_bounds__(NT, 2) k_fgp_pair(PairArgs a, Dims d, int zc, const StopCtl* ctl) {
    extern __shared__ float ring[];  // [RING][NIN][NT]
    __shared__ float sR1[NT], sR2[NT], sQ1[NT], sQ2[NT];  // R^k and R^{k+1} x/y components
    __shared__ float sU[2][NT], sV[2][NT];                // U^k and U^{k+1}, two planes each
    if (ctl->stop) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int oc = ty * BX + tx;
    const int nx = d.nx, ny = d.ny, nz = d.nz;
    const int x = blockIdx.x * OX + tx - 2;
    const int y = blockIdx.y * OY + ty - 2;
    const int z0 = blockIdx.z * zc;
    const int z1 = min(z0 + zc, nz);
    const bool in_xy = (x >= 0) && (x < nx) && (y >= 0) && (y < ny);
    const bool u1_pt = in_xy && tx >= 1 && ty >= 1;
    const bool p1_pt = u1_pt && tx <= BX - 2 && ty <= BY - 2;  // P^k valid (inner 30 x 14)
    const bool u2_pt = in_xy && tx >= 2 && ty >= 2 && tx <= BX - 2 && ty <= BY - 2;
    const bool o_pt = u2_pt && tx <= BX - 3 && ty <= BY - 3;   // written (inner 28 x 12)
    const IT col = (IT)min(max(y, 0), ny - 1) * nx + min(max(x, 0), nx - 1);
    const IT sxy = (IT)d.sxy;
    const float* src[NIN] = {a.pc[0], a.pc[1], a.pc[2], a.po[0], a.po[1], a.po[2], a.f};

    auto issue = [&](int k, int slot) {
        const bool valid = in_xy && k >= 0 && k < nz;
        const IT v = (IT)min(max(k, 0), nz - 1) * sxy + col;
        float* dst = ring + (size_t)slot * NIN * NT + oc;
#pragma unroll
        for (int q = 0; q < NIN; q++) cp_async4_zfill(dst + q * NT, src[q] + v, valid);
        cp_async_commit_group();
    };
    auto rd = [&](int slot, int q) -> float { return ring[((size_t)slot * NIN + q) * NT + oc]; };

    // ring slot of plane j is sj; planes z0-2 .. z0-2+AHEAD-1 in flight first
    int sj = 0;
    for (int t = 0; t < AHEAD; t++) issue(z0 - 2 + t, t);

    // level 1 state: R^k of plane j-1, U^k of plane j-1, P^k of plane j-1 (for level 2)
    float r1p = 0.f, r2p = 0.f, r3p = 0.f, up = 0.f;
    float q1k = 0.f, q2k = 0.f, q3k = 0.f;  // P^k(j-2) handed to level 2 (formed one step earlier)
    // level 2 state: R^{k+1} and U^{k+1} of plane j-3
    float s1p = 0.f, s2p = 0.f, s3p = 0.f, vp = 0.f;

    auto step = [&](auto par, int j) {
        constexpr int PJ = decltype(par)::value;  // parity slot of plane j (and j-2)
        // copies of plane j+AHEAD; wait for this thread's copies of plane j
        {
            int s = sj + AHEAD;
            if (s >= RING) s -= RING;
            issue(j + AHEAD, s);
        }
        cp_async_wait_group<AHEAD>();
        int s2 = sj - 2;
        if (s2 < 0) s2 += RING;
        // A. level 1: R^k(j); level 2: R^{k+1}(j-2) from P^k(j-2) and P^{k-1}(j-2)
        const float c1v = rd(sj, 0), c2v = rd(sj, 1), c3v = rd(sj, 2);
        const float r1 = c1v + a.c1 * (c1v - rd(sj, 3));
        const float r2 = c2v + a.c1 * (c2v - rd(sj, 4));
        const float r3 = c3v + a.c1 * (c3v - rd(sj, 5));
        const float fj = rd(sj, 6);
        const float b1v = rd(s2, 0), b2v = rd(s2, 1), b3v = rd(s2, 2);
        const float t1 = q1k + a.c2 * (q1k - b1v);
        const float t2 = q2k + a.c2 * (q2k - b2v);
        const float t3 = q3k + a.c2 * (q3k - b3v);
        const float fm = rd(s2, 6);
        sR1[oc] = r1;
        sR2[oc] = r2;
        sQ1[oc] = t1;
        sQ2[oc] = t2;
        __syncthreads();
        // B. U^k(j) and U^{k+1}(j-2)
        float u = 0.f;
        if (u1_pt && j >= 0 && j < nz) {
            const float s = r1 + r2 + r3 - sR1[oc - 1] - sR2[oc - BX] - r3p;
            u = fj - a.lam * s;
            if (a.nonneg && u < 0.f) u = 0.f;
        }
        const int m = j - 2;
        float v = 0.f;
        if (u2_pt && m >= 0 && m < nz) {
            const float s = t1 + t2 + t3 - sQ1[oc - 1] - sQ2[oc - BX] - s3p;
            v = fm - a.lam * s;
            if (a.nonneg && v < 0.f) v = 0.f;
            if (a.write_u2 && o_pt && m >= z0 && m < z1) a.u[(IT)m * sxy + col] = v;
        }
        sU[PJ][oc] = u;
        sV[PJ][oc] = v;
        __syncthreads();
        // C. level 1: P^k(j-1); level 2: P^{k+1}(j-3)
        const int kp = j - 1;
        float n1 = 0.f, n2 = 0.f, n3 = 0.f;
        if (p1_pt && kp >= 0 && kp < nz) {
            const float g1 = (x == nx - 1) ? 0.f : up - sU[1 - PJ][oc + 1];
            const float g2 = (y == ny - 1) ? 0.f : up - sU[1 - PJ][oc + BX];
            const float g3 = (kp != nz - 1) ? up - u : 0.f;
            p_update(r1p, r2p, r3p, g1, g2, g3, a.multip, a.aniso, n1, n2, n3);
            if (o_pt && kp >= z0 && kp < z1) {
                const IT o = (IT)kp * sxy + col;
                a.pn1[0][o] = n1;
                a.pn1[1][o] = n2;
                a.pn1[2][o] = n3;
            }
        }
        const int mp = j - 3;
        if (a.write_p2 && o_pt && mp >= z0 && mp < z1) {
            const float g1 = (x == nx - 1) ? 0.f : vp - sV[1 - PJ][oc + 1];
            const float g2 = (y == ny - 1) ? 0.f : vp - sV[1 - PJ][oc + BX];
            const float g3 = (mp != nz - 1) ? vp - v : 0.f;
            float p1, p2, p3;
            p_update(s1p, s2p, s3p, g1, g2, g3, a.multip, a.aniso, p1, p2, p3);
            const IT o = (IT)mp * sxy + col;
            a.pn2[0][o] = p1;
            a.pn2[1][o] = p2;
            a.pn2[2][o] = p3;
        }
        r1p = r1;
        r2p = r2;
        r3p = r3;
        up = u;
        q1k = n1;
        q2k = n2;
        q3k = n3;
        s1p = t1;
        s2p = t2;
        s3p = t3;
        vp = v;
        sj = (sj + 1 == RING) ? 0 : sj + 1;
    };
    int j = z0 - 2;
    for (; j + 1 <= z1 + 2; j += 2) {
        step(Ic<0>{}, j);
        step(Ic<1>{}, j + 1);
    }
    if (j <= z1 + 2) step(Ic<0>{}, j);
    cp_async_wait_group<0>();  // no copy outlives the CTA
}

}  // namespace

PairPlan fgp_pair_plan(const Dims& d) {
    PairPlan T;
    // opt-in (CILREG_FGP_PAIR=1): on GB300 a pair takes 1.3x the time of two
    // single iterations (instruction- and barrier-bound at two CTAs per SM),
    // although it moves 52 B per voxel instead of 80
    const char* e = getenv("CILREG_FGP_PAIR");
    T.use = d.nz > 1 && e && e[0] == '1';
    if (!T.use) return T;
    static const bool attr_ok = [] {
        bool ok = cudaFuncSetAttribute(k_fgp_pair<int>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)RING_BYTES) == cudaSuccess;
        ok = ok && cudaFuncSetAttribute(k_fgp_pair<long long>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)RING_BYTES) == cudaSuccess;
        cudaGetLastError();
        return ok;
    }();
    if (!attr_ok) {
        T.use = false;
        return T;
    }
    static const int resident = [] {
        int r = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&r, k_fgp_pair<int>, NT, RING_BYTES) != cudaSuccess ||
            r <= 0)
            r = 1;
        cudaGetLastError();
        return r;
    }();
    T.block = dim3(BX, BY, 1);
    const long long tiles = (long long)((d.nx + OX - 1) / OX) * ((d.ny + OY - 1) / OY);
    T.zchunk = wave_zchunk(tiles, d.nz, resident, 5, ZCHUNK);
    T.grid = dim3((d.nx + OX - 1) / OX, (d.ny + OY - 1) / OY, (d.nz + T.zchunk - 1) / T.zchunk);
    T.nblocks = (long long)T.grid.x * T.grid.y * T.grid.z;
    return T;
}

int fgp_pair_step(const PairPlan& T, const float* const pc[3], const float* const po[3], float* const pn1[3],
                  float* const pn2[3], const float* f, float* u, float lam, float c1, float c2, float multip,
                  int nonneg, int aniso, int write_u2, int write_p2, const Dims& d, const StopCtl* ctl,
                  cudaStream_t s) {
    PairArgs a;
    for (int i = 0; i < 3; i++) {
        a.pc[i] = pc[i];
        a.po[i] = po[i];
        a.pn1[i] = pn1[i];
        a.pn2[i] = pn2[i];
    }
    a.f = f;
    a.u = u;
    a.lam = lam;
    a.c1 = c1;
    a.c2 = c2;
    a.multip = multip;
    a.nonneg = nonneg;
    a.aniso = aniso;
    a.write_u2 = write_u2;
    a.write_p2 = write_p2;
    if (d.n < (1LL << 31))
        k_fgp_pair<int><<<T.grid, T.block, RING_BYTES, s>>>(a, d, T.zchunk, ctl);
    else
        k_fgp_pair<long long><<<T.grid, T.block, RING_BYTES, s>>>(a, d, T.zchunk, ctl);
    CILREG_CUDA(cudaGetLastError());
    return OK;
}

}  // namespace cilreg
