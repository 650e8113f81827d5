// Hand-written adjoint (vector-Jacobian product) of the unrolled FGP-TV
// iteration, with checkpointed recomputation.
//
// Forward (FGP_TV_core.c:40-269, epsil = 0, L iterations), iteration k:
//   R_k = P_{k-1} + c_k (P_{k-1} - P_{k-2})         (P_{-1} = P_{-2} = 0)
//   Z_k = f - lambda A R_k,   A R = sum_c (R_c - R_c[-e_c]),  R_c[-1] = 0
//   U_k = max(Z_k, 0) when nonneg, else Z_k
//   Q_k = R_k + m B U_k,      (B U)_c = U - U[+e_c] (0 at the last index), m = 1/(12 lambda) (1/(8 lambda) in 2D)
//   P_k = proj(Q_k)           (iso: Q / max(1, |Q|); aniso: per component)
// and the output is y = U_{L-1}.  Given ybar = dL/dy, the reverse sweep is
//   Pbar_k = (1 + c_{k+1}) Rbar_{k+1} - c_{k+2} Rbar_{k+2}
//   Qbar_k = J_proj(Q_k)^T Pbar_k
//   Zbar_k = 1[Z_k >= 0] * (m B^T Qbar_k + [k == L-1] ybar)
//   fbar  += Zbar_k
//   lambar += -<Zbar_k, A R_k> + (dm/dlambda) <Qbar_k, B U_k>
//   Rbar_k = Qbar_k - lambda A^T Zbar_k,  (A^T Z)_c = Z - Z[+e_c] (0 past the last index)
// Four kernels per reverse iteration: Z_k and A R_k once per voxel, then
// Qbar, Zbar, Rbar.  The forward states
// are stored every `ckpt` iterations and each segment is recomputed with the
// production iteration kernel before its reverse sweep, so the linearisation
// point is exactly the forward pass the caller saw.
#include <math.h>

#include <vector>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "fgp_tiled.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

struct AdjArgs {
    const float* pm1[3];  // P_{k-1}
    const float* pm2[3];  // P_{k-2}
    const float* f;
    const float* ybar;    // only on the last iteration
    const float* rb1[3];  // Rbar_{k+1}
    const float* rb2[3];  // Rbar_{k+2}
    float* qb[3];         // Qbar_k (out of kernel a)
    float* zb;            // Zbar_k (out of kernel b)
    float* fbar;          // accumulated
    float* rb0[3];        // Rbar_k (out of kernel c)
    float* zz;            // Z_k = f - lambda A R_k (before the clamp; kernel u)
    float* ar;            // A R_k (kernel u)
    float lam, m, ck, a1, a2;
    int nonneg, aniso;
};

template <bool THREE>
__device__ __forceinline__ float r_at(const AdjArgs& a, int c, long long v) {
    const float p = ldg(a.pm1[c], v);
    return p + a.ck * (p - ldg(a.pm2[c], v));
}

// A R at (i,j,k) (the divergence term of the objective step)
template <bool THREE>
__device__ __forceinline__ float ar_at(const AdjArgs& a, const Dims& d, int i, int j, int k) {
    const long long v = vid(d, i, j, k);
    const float b1 = (i == 0) ? 0.f : r_at<THREE>(a, 0, v - 1);
    const float b2 = (j == 0) ? 0.f : r_at<THREE>(a, 1, v - d.nx);
    if (THREE) {
        const float b3 = (k == 0) ? 0.f : r_at<THREE>(a, 2, v - d.sxy);
        return r_at<THREE>(a, 0, v) + r_at<THREE>(a, 1, v) + r_at<THREE>(a, 2, v) - b1 - b2 - b3;
    }
    return r_at<THREE>(a, 0, v) + r_at<THREE>(a, 1, v) - b1 - b2;
}

#define ADJ_LOOP_BEGIN                                       \
    const int i = blockIdx.x * 32 + threadIdx.x;             \
    const int j = blockIdx.y * 8 + threadIdx.y;              \
    const int k0 = blockIdx.z * kz;                          \
    float acc = 0.f;                                         \
    if (i < d.nx && j < d.ny) {                              \
        for (int kk = 0; kk < kz; kk++) {                    \
            const int k = k0 + kk;                           \
            if (k >= d.nz) break;                            \
            const long long v = vid(d, i, j, k);

#define ADJ_LOOP_END \
    }                \
    }

// u: Z_k = f - lambda A R_k (the objective step before the clamp) and A R_k,
// once per voxel (same expressions as u_at)
template <bool THREE>
__global__ void __launch_bounds__(256) k_adj_u(AdjArgs a, Dims d, int kz) {
    ADJ_LOOP_BEGIN
    const float ar = ar_at<THREE>(a, d, i, j, k);
    a.ar[v] = ar;
    a.zz[v] = ldg(a.f, v) - a.lam * ar;
    ADJ_LOOP_END
    (void)acc;
}

__device__ __forceinline__ float clamp_u(const AdjArgs& a, float z) { return (a.nonneg && z < 0.f) ? 0.f : z; }

// a: Qbar_k = J^T Pbar_k, and <Qbar_k, B U_k> into the partials
template <bool THREE>
__global__ void __launch_bounds__(256) k_adj_q(AdjArgs a, Dims d, int kz, double2* partials) {
    ADJ_LOOP_BEGIN
    const float u = clamp_u(a, ldg(a.zz, v));
    float bu[3] = {0.f, 0.f, 0.f};
    bu[0] = (i == d.nx - 1) ? 0.f : u - clamp_u(a, ldg(a.zz, v + 1));
    bu[1] = (j == d.ny - 1) ? 0.f : u - clamp_u(a, ldg(a.zz, v + d.nx));
    if (THREE) bu[2] = (k == d.nz - 1) ? 0.f : u - clamp_u(a, ldg(a.zz, v + d.sxy));
    const int nc = THREE ? 3 : 2;
    float q[3], pb[3], qb[3];
    for (int c = 0; c < 3; c++) {
        q[c] = 0.f;
        pb[c] = 0.f;
    }
    for (int c = 0; c < nc; c++) {
        q[c] = r_at<THREE>(a, c, v) + a.m * bu[c];
        pb[c] = a.a1 * ldg(a.rb1[c], v) - a.a2 * ldg(a.rb2[c], v);
    }
    if (!a.aniso) {
        const float den = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        if (den > 1.f) {
            const float inv = 1.f / sqrtf(den);
            const float dot = (q[0] * pb[0] + q[1] * pb[1] + q[2] * pb[2]) * inv;
            for (int c = 0; c < 3; c++) qb[c] = (pb[c] - q[c] * inv * dot) * inv;
        } else {
            for (int c = 0; c < 3; c++) qb[c] = pb[c];
        }
    } else {
        for (int c = 0; c < 3; c++) qb[c] = (fabsf(q[c]) < 1.f) ? pb[c] : 0.f;
    }
    for (int c = 0; c < nc; c++) {
        a.qb[c][v] = qb[c];
        acc += qb[c] * bu[c];
    }
    ADJ_LOOP_END
    block_pair_partial<256>(acc, 0.f, partials, block_slot());
}

// b: Zbar_k = mask (m B^T Qbar_k + ybar); fbar += Zbar; -<Zbar, A R_k> into the partials
template <bool THREE>
__global__ void __launch_bounds__(256) k_adj_z(AdjArgs a, Dims d, int kz, double2* partials) {
    ADJ_LOOP_BEGIN
    float w = ((i < d.nx - 1) ? ldg(a.qb[0], v) : 0.f) - ((i >= 1) ? ldg(a.qb[0], v - 1) : 0.f);
    w += ((j < d.ny - 1) ? ldg(a.qb[1], v) : 0.f) - ((j >= 1) ? ldg(a.qb[1], v - d.nx) : 0.f);
    if (THREE) w += ((k < d.nz - 1) ? ldg(a.qb[2], v) : 0.f) - ((k >= 1) ? ldg(a.qb[2], v - d.sxy) : 0.f);
    w = a.m * w;
    if (a.ybar) w += ldg(a.ybar, v);
    const float ar = ldg(a.ar, v);
    const float z = ldg(a.zz, v);
    const float zb = (a.nonneg && z < 0.f) ? 0.f : w;
    a.zb[v] = zb;
    a.fbar[v] += zb;
    acc += -zb * ar;
    ADJ_LOOP_END
    block_pair_partial<256>(acc, 0.f, partials, block_slot());
}

// c: Rbar_k = Qbar_k - lambda A^T Zbar_k
template <bool THREE>
__global__ void __launch_bounds__(256) k_adj_r(AdjArgs a, Dims d, int kz) {
    ADJ_LOOP_BEGIN
    const float z = ldg(a.zb, v);
    a.rb0[0][v] = ldg(a.qb[0], v) - a.lam * (z - ((i + 1 < d.nx) ? ldg(a.zb, v + 1) : 0.f));
    a.rb0[1][v] = ldg(a.qb[1], v) - a.lam * (z - ((j + 1 < d.ny) ? ldg(a.zb, v + d.nx) : 0.f));
    if (THREE) a.rb0[2][v] = ldg(a.qb[2], v) - a.lam * (z - ((k + 1 < d.nz) ? ldg(a.zb, v + d.sxy) : 0.f));
    ADJ_LOOP_END
    (void)acc;
}

// add the .x of every partial into acc[slot] (FP64, one CTA, fixed order)
__global__ void __launch_bounds__(1024) k_accumulate(const double2* part, long long n, double* acc, int slot) {
    double s = 0.0;
    for (long long p = threadIdx.x; p < n; p += 1024) s += part[p].x;
    __shared__ double sh[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = warp_sum(sh[threadIdx.x]);
        if (threadIdx.x == 0) acc[slot] += s;
    }
}

}  // namespace

int fgp_vjp_run(const float* f, const float* ybar, float lam, int iters, int methodTV, int nonneg, int ckpt,
                const Dims& d, cudaStream_t s, float* fbar, double* lambar) {
    CILREG_RANGE("cilreg FGP-TV adjoint");
    if (iters < 1) return fail(ERR_ARG, __FILE__, __LINE__, "the unrolled map needs at least one iteration");
    if (ckpt < 1) ckpt = 1;
    const bool three = d.nz > 1;
    const int nc = three ? 3 : 2;
    const long long n = d.n;
    const int L = iters;
    // coefficients: iteration k forms R_k with cc[k] (cc[0] = 0), FGP_TV_core.c:138-139
    std::vector<float> cc(L + 3, 0.0f);
    {
        float tk = 1.0f, cprev = 0.0f;
        for (int k = 0; k < L + 3; k++) {
            cc[k] = cprev;
            const float tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
            cprev = (tk - 1.0f) / tkp1;
            tk = tkp1;
        }
    }
    const float m = three ? (1.0f / (12.0f * lam)) : (1.0f / (8.0f * lam));
    const double dm = three ? -1.0 / (12.0 * (double)lam * lam) : -1.0 / (8.0 * (double)lam * lam);

    Scratch sc(s);
    const int nseg = (L + ckpt - 1) / ckpt;
    auto arr = [&](long long count) { return sc.floats(count); };
    // checkpoints: (P_{k0-1}, P_{k0-2}) per segment start k0
    std::vector<float*> ck_pm1(nseg * 3, nullptr), ck_pm2(nseg * 3, nullptr);
    for (int g = 0; g < nseg; g++)
        for (int c = 0; c < nc; c++) {
            ck_pm1[3 * g + c] = arr(n);
            ck_pm2[3 * g + c] = arr(n);
            if (!ck_pm1[3 * g + c] || !ck_pm2[3 * g + c]) return sc.status();
        }
    // forward ring, segment store (P_k of the segment), adjoint ring
    float* ring[3][3] = {};
    float* seg[64][3] = {};
    float* rbar[3][3] = {};
    float* qb[3] = {};
    if (ckpt > 64) return fail(ERR_ARG, __FILE__, __LINE__, "checkpoint interval %d above 64", ckpt);
    for (int c = 0; c < nc; c++) {
        for (int r = 0; r < 3; r++) {
            ring[r][c] = arr(n);
            rbar[r][c] = arr(n);
            if (!ring[r][c] || !rbar[r][c]) return sc.status();
        }
        for (int q = 0; q < ckpt; q++) {
            seg[q][c] = arr(n);
            if (!seg[q][c]) return sc.status();
        }
        qb[c] = arr(n);
        if (!qb[c]) return sc.status();
    }
    float* zb = arr(n);
    float* zz = arr(n);
    float* arv = arr(n);
    StopCtl* ctl = (StopCtl*)sc.bytes(sizeof(StopCtl));
    double* acc = (double*)sc.bytes(2 * sizeof(double));
    const Launch3 LA = plan_launch(d);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)num_blocks(LA));
    if (!zb || !zz || !arv || !ctl || !acc || !part) return sc.status();
    CILREG_TRY(launch_init_ctl(ctl, iters, s));
    CILREG_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s));
    CILREG_CUDA(cudaMemsetAsync(fbar, 0, sizeof(float) * n, s));
    const size_t nb = sizeof(float) * (size_t)n;
    const TiledPlan T = fgp_tiled_plan(d);

    // one production forward iteration k from (pm1, pm2) into pn
    auto fwd = [&](int k, float* const pm1[3], float* const pm2[3], float* const pn[3]) -> int {
        const float* pc[3] = {pm1[0], pm1[1], pm1[2]};
        const float* po[3] = {pm2[0], pm2[1], pm2[2]};
        CILREG_TRY(fgp_tiled_step(T, pc, po, pn, f, nullptr, lam, cc[k], m, nonneg == 1, methodTV != 0, 0, 1, 0, d,
                                  ctl, nullptr, s));
        note_launch();
        return OK;
    };

    // pass 1: forward, storing (P_{k0-1}, P_{k0-2}) at every segment start
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < nc; c++) CILREG_CUDA(cudaMemsetAsync(ring[r][c], 0, nb, s));
    for (int k = 0; k < L - 1; k++) {
        float* pm1[3] = {ring[(k + 2) % 3][0], ring[(k + 2) % 3][1], ring[(k + 2) % 3][2]};
        float* pm2[3] = {ring[(k + 1) % 3][0], ring[(k + 1) % 3][1], ring[(k + 1) % 3][2]};
        if (k % ckpt == 0)
            for (int c = 0; c < nc; c++) {
                CILREG_CUDA(cudaMemcpyAsync(ck_pm1[3 * (k / ckpt) + c], pm1[c], nb, cudaMemcpyDeviceToDevice, s));
                CILREG_CUDA(cudaMemcpyAsync(ck_pm2[3 * (k / ckpt) + c], pm2[c], nb, cudaMemcpyDeviceToDevice, s));
            }
        float* pn[3] = {ring[k % 3][0], ring[k % 3][1], ring[k % 3][2]};
        CILREG_TRY(fwd(k, pm1, pm2, pn));
    }
    if ((L - 1) % ckpt == 0) {  // the last segment starts at the last iteration
        const int k = L - 1;
        for (int c = 0; c < nc; c++) {
            CILREG_CUDA(cudaMemcpyAsync(ck_pm1[3 * (k / ckpt) + c], ring[(k + 2) % 3][c], nb, cudaMemcpyDeviceToDevice, s));
            CILREG_CUDA(cudaMemcpyAsync(ck_pm2[3 * (k / ckpt) + c], ring[(k + 1) % 3][c], nb, cudaMemcpyDeviceToDevice, s));
        }
    }

    // reverse sweep; Rbar_L = Rbar_{L+1} = 0
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < nc; c++) CILREG_CUDA(cudaMemsetAsync(rbar[r][c], 0, nb, s));
    for (int g = nseg - 1; g >= 0; g--) {
        const int k0 = g * ckpt, k1 = (k0 + ckpt < L) ? k0 + ckpt : L;
        float* cp1[3] = {ck_pm1[3 * g], ck_pm1[3 * g + 1], ck_pm1[3 * g + 2]};
        float* cp2[3] = {ck_pm2[3 * g], ck_pm2[3 * g + 1], ck_pm2[3 * g + 2]};
        // recompute P_k for k in [k0, k1-1) into seg[k - k0]
        auto P = [&](int k, int c) -> float* {  // P_k for k >= k0 - 2
            if (k >= k0) return seg[k - k0][c];
            return (k == k0 - 1) ? cp1[c] : cp2[c];
        };
        for (int k = k0; k < k1 - 1; k++) {
            float* pm1[3] = {P(k - 1, 0), P(k - 1, 1), P(k - 1, 2)};
            float* pm2[3] = {P(k - 2, 0), P(k - 2, 1), P(k - 2, 2)};
            float* pn[3] = {seg[k - k0][0], seg[k - k0][1], seg[k - k0][2]};
            if (nc == 2) pm1[2] = pm2[2] = pn[2] = nullptr;
            CILREG_TRY(fwd(k, pm1, pm2, pn));
        }
        for (int k = k1 - 1; k >= k0; k--) {
            AdjArgs a;
            for (int c = 0; c < 3; c++) {
                a.pm1[c] = (c < nc) ? P(k - 1, c) : nullptr;
                a.pm2[c] = (c < nc) ? P(k - 2, c) : nullptr;
                a.rb1[c] = rbar[(k + 1) % 3][c];
                a.rb2[c] = rbar[(k + 2) % 3][c];
                a.rb0[c] = rbar[k % 3][c];
                a.qb[c] = qb[c];
            }
            a.f = f;
            a.ybar = (k == L - 1) ? ybar : nullptr;
            a.zb = zb;
            a.zz = zz;
            a.ar = arv;
            a.fbar = fbar;
            a.lam = lam;
            a.m = m;
            a.ck = cc[k];
            a.a1 = 1.0f + cc[k + 1];
            a.a2 = cc[k + 2];
            a.nonneg = (nonneg == 1);
            a.aniso = (methodTV != 0);
            if (three) {
                k_adj_u<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
                k_adj_q<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc, 0);
                k_adj_z<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc, 1);
                k_adj_r<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
            } else {
                k_adj_u<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
                k_adj_q<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc, 0);
                k_adj_z<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc, 1);
                k_adj_r<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
            }
            CILREG_CUDA(cudaGetLastError());
            note_launch(6);
        }
    }
    double h[2] = {0.0, 0.0};
    CILREG_CUDA(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (lambar) *lambar = h[1] + dm * h[0];
    return OK;
}

}  // namespace cilreg

using namespace cilreg;

extern "C" int cilreg_fgp_tv_vjp_dev(const float* d_in, const float* d_ybar, float* d_inbar, double* lambar,
                                     float lambdaPar, int iters, int methodTV, int nonneg, int checkpoint, int dimX,
                                     int dimY, int dimZ, void* stream) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    if (!d_in || !d_ybar || !d_inbar) return fail(ERR_ARG, __FILE__, __LINE__, "null device pointer");
    if (!(lambdaPar > 0.0f)) return fail(ERR_ARG, __FILE__, __LINE__, "lambda must be positive");
    return fgp_vjp_run(d_in, d_ybar, lambdaPar, iters, methodTV, nonneg, checkpoint,
                       make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ), (cudaStream_t)stream, d_inbar, lambar);
}
