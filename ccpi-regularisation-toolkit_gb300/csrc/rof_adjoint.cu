// Hand-written adjoint (vector-Jacobian product) of the unrolled ROF-TV
// iteration, with checkpointed recomputation.
//
// Forward (ROF_TV_core.c:50-317, scalar lambda, no stopping rule), U_0 = f:
//   U_{k+1} = U_k + tau (lambda div D(U_k) - (U_k - f)),
//   div D(v) = sum_a D_a(v) - D_a(lo_a(v)),
//   D_a(u)   = p_a / sqrt(p_a^2 + sum_{b != a} m_b^2 + 1e-8),
//   p_b = U(hi_b(u)) - U(u),  q_b = U(u) - U(lo_b(u)),  m_b = minmod(p_b, q_b),
// with hi/lo the mirrored neighbours (i+1 -> i-1 at the last index, i-1 ->
// i+1 at the first, an axis of length 1 maps to itself), and y = U_L.
//
// Reverse step, given W = Ubar_{k+1}:
//   Ubar_k = (1 - tau) W + tau lambda J_divD(U_k)^T W,   fbar += tau W,
//   lambar += tau <W, div D(U_k)>,                        and fbar += Ubar_0.
// Transposing the divergence, <W, div D> = sum_a sum_u Wa(u) D_a(u) with
//   Wa(u) = W(u) - sum_{v : lo_a(v) = u} W(v).
// D_a(u) depends on U through p_a and, for b != a, through the one of p_b,
// q_b that minmod selects (derivative 1 on the smaller magnitude when both
// have the same strict sign, 0 otherwise).  Collecting the terms by the axis
// of the difference they enter:
//   E_c(u): coefficient of (U(hi_c(u)) - U(u)),  F_c(u): of (U(u) - U(lo_c(u))),
//   E_c += Wa dD_a/dp_c (c = a, or c != a with p_c selected), F_c += Wa dD_a/dq_c,
//   dD_a/dp_a = (S - p_a^2) / S^1.5,  dD_a/dm_b = -p_a m_b / S^1.5,
// and the transpose is the gather
//   (J^T W)(v) = sum_c [ sum_{u : hi_c(u) = v} E_c(u) - E_c(v) + F_c(v) - sum_{u : lo_c(u) = v} F_c(u) ].
// Two kernels per reverse iteration: coefficients (E, F and the lambda term)
// and the gather.  The forward states are stored every `ckpt` iterations and
// each segment is recomputed with the production iteration kernel, so the
// linearisation point is exactly the forward pass the caller saw.
#include <math.h>

#include <vector>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

struct RofAdjArgs {
    const float* u;   // U_k (linearisation point)
    const float* w;   // Ubar_{k+1}
    float* e[3];      // E_c
    float* fq[3];     // F_c
    float* ubar;      // Ubar_k (gather output)
    float* fbar;      // accumulated
    float lam, tau;
};

// positions u along one axis with hi(u) = p / lo(u) = p (at most two)
__device__ __forceinline__ int hi_pre(int p, int n, int* q) {
    if (n == 1) { q[0] = p; return 1; }
    int c = 0;
    if (p >= 1) q[c++] = p - 1;
    if (p == n - 2) q[c++] = p + 1;
    return c;
}
__device__ __forceinline__ int lo_pre(int p, int n, int* q) {
    if (n == 1) { q[0] = p; return 1; }
    int c = 0;
    if (p <= n - 2) q[c++] = p + 1;
    if (p == 1) q[c++] = p - 1;
    return c;
}

// offset of the voxel at coordinate `q` along axis `ax` from (i, j, k)
__device__ __forceinline__ long long at_axis(const Dims& d, int i, int j, int k, int ax, int q) {
    return ax == 0 ? vid(d, q, j, k) : (ax == 1 ? vid(d, i, q, k) : vid(d, i, j, q));
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_rof_adj_coef(RofAdjArgs a, Dims d, int kz, double2* partials) {
    constexpr int NC = THREE ? 3 : 2;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    float acc = 0.f;
    if (i < d.nx && j < d.ny) {
        for (int kk = 0; kk < kz; kk++) {
            const int k = k0 + kk;
            if (k >= d.nz) break;
            const long long v = vid(d, i, j, k);
            const int pos[3] = {i, j, k};
            const int ext[3] = {d.nx, d.ny, d.nz};
            const float c = ldg(a.u, v);
            float p[3], q[3], m[3];
            bool selp[3], selq[3];
            for (int b = 0; b < NC; b++) {
                p[b] = ldg(a.u, at_axis(d, i, j, k, b, nb_hi(pos[b], ext[b]))) - c;
                q[b] = c - ldg(a.u, at_axis(d, i, j, k, b, nb_lo(pos[b], ext[b])));
                const bool same = (p[b] > 0.f && q[b] > 0.f) || (p[b] < 0.f && q[b] < 0.f);
                const bool pmin = fabsf(p[b]) < fabsf(q[b]);
                m[b] = same ? (pmin ? p[b] : q[b]) : 0.f;
                selp[b] = same && pmin;
                selq[b] = same && !pmin;
            }
            const float wv = ldg(a.w, v);
            float E[3] = {0.f, 0.f, 0.f}, F[3] = {0.f, 0.f, 0.f};
            for (int ax = 0; ax < NC; ax++) {
                int qq[2];
                const int nq = lo_pre(pos[ax], ext[ax], qq);
                float wa = wv;
                for (int t = 0; t < nq; t++) wa -= ldg(a.w, at_axis(d, i, j, k, ax, qq[t]));
                float rest = 1.0e-8f;
                for (int b = 0; b < NC; b++)
                    if (b != ax) rest += m[b] * m[b];
                const float S = p[ax] * p[ax] + rest;
                const float T = sqrtf(S);
                const float inv = 1.0f / (S * T);
                acc += wa * (p[ax] / T);
                E[ax] += wa * rest * inv;
                for (int b = 0; b < NC; b++) {
                    if (b == ax) continue;
                    const float g = -wa * p[ax] * m[b] * inv;
                    if (selp[b]) E[b] += g;
                    if (selq[b]) F[b] += g;
                }
            }
            for (int b = 0; b < NC; b++) {
                a.e[b][v] = E[b];
                a.fq[b][v] = F[b];
            }
        }
    }
    block_pair_partial<256>(acc, 0.f, partials, block_slot());
}

template <bool THREE>
__global__ void __launch_bounds__(256) k_rof_adj_gather(RofAdjArgs a, Dims d, int kz) {
    constexpr int NC = THREE ? 3 : 2;
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k0 = blockIdx.z * kz;
    if (i >= d.nx || j >= d.ny) return;
    for (int kk = 0; kk < kz; kk++) {
        const int k = k0 + kk;
        if (k >= d.nz) break;
        const long long v = vid(d, i, j, k);
        const int pos[3] = {i, j, k};
        const int ext[3] = {d.nx, d.ny, d.nz};
        float g = 0.f;
        for (int ax = 0; ax < NC; ax++) {
            int qq[2];
            int nq = hi_pre(pos[ax], ext[ax], qq);
            for (int t = 0; t < nq; t++) g += ldg(a.e[ax], at_axis(d, i, j, k, ax, qq[t]));
            g += ldg(a.fq[ax], v) - ldg(a.e[ax], v);
            nq = lo_pre(pos[ax], ext[ax], qq);
            for (int t = 0; t < nq; t++) g -= ldg(a.fq[ax], at_axis(d, i, j, k, ax, qq[t]));
        }
        const float wv = ldg(a.w, v);
        a.ubar[v] = (1.0f - a.tau) * wv + a.tau * a.lam * g;
        a.fbar[v] += a.tau * wv;
    }
}

// acc[0] += sum of the partials' .x (FP64, one CTA, fixed order)
__global__ void __launch_bounds__(1024) k_rof_adj_accumulate(const double2* part, long long n, double* acc) {
    double s = 0.0;
    for (long long t = threadIdx.x; t < n; t += 1024) s += part[t].x;
    __shared__ double sh[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = warp_sum(sh[threadIdx.x]);
        if (threadIdx.x == 0) acc[0] += s;
    }
}

__global__ void k_rof_adj_add(float* __restrict__ dst, const float* __restrict__ src, long long n) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; t < n; t += stride) dst[t] += src[t];
}

}  // namespace

int rof_vjp_run(const float* f, const float* ybar, float lam, int iters, float tau, int ckpt, const Dims& d,
                cudaStream_t s, float* fbar, double* lambar) {
    CILREG_RANGE("cilreg ROF-TV adjoint");
    if (iters < 1) return fail(ERR_ARG, __FILE__, __LINE__, "the unrolled map needs at least one iteration");
    if (ckpt < 1) return fail(ERR_ARG, __FILE__, __LINE__, "checkpoint interval %d below 1", ckpt);
    if (ckpt > iters) ckpt = iters;
    const bool three = d.nz > 1;
    const int nc = three ? 3 : 2;
    const long long n = d.n;
    const size_t nb = sizeof(float) * (size_t)n;
    const int L = iters;
    const int nseg = (L + ckpt - 1) / ckpt;

    Scratch sc(s);
    // U_{g ckpt} for every segment g >= 1 (segment 0 starts from f)
    std::vector<float*> ck(nseg, nullptr);
    for (int g = 1; g < nseg; g++)
        if (!(ck[g] = sc.floats(n))) return sc.status();
    // states U_{k0+1} .. U_{k0+ckpt-1} of the segment being reversed
    std::vector<float*> seg(ckpt, nullptr);
    for (int q = 1; q < ckpt; q++)
        if (!(seg[q] = sc.floats(n))) return sc.status();
    float* E[3] = {};
    float* Fq[3] = {};
    for (int c = 0; c < nc; c++)
        if (!(E[c] = sc.floats(n)) || !(Fq[c] = sc.floats(n))) return sc.status();
    float* wb[2] = {sc.floats(n), sc.floats(n)};
    float* ping[2] = {sc.floats(n), sc.floats(n)};
    StopCtl* ctl = (StopCtl*)sc.bytes(sizeof(StopCtl));
    double* acc = (double*)sc.bytes(sizeof(double));
    const Launch3 LA = plan_launch(d);
    double2* part = (double2*)sc.bytes(sizeof(double2) * (size_t)num_blocks(LA));
    if (!wb[0] || !wb[1] || !ping[0] || !ping[1] || !ctl || !acc || !part) return sc.status();
    CILREG_TRY(launch_init_ctl(ctl, iters, s));
    CILREG_CUDA(cudaMemsetAsync(acc, 0, sizeof(double), s));
    CILREG_CUDA(cudaMemsetAsync(fbar, 0, nb, s));

    // pass 1: forward from f up to the last segment start, keeping U there
    // and at every earlier segment start
    const float* cur = f;
    for (int k = 0; k < (nseg - 1) * ckpt; k++) {
        float* nxt = ((k + 1) % ckpt == 0) ? ck[(k + 1) / ckpt] : ping[k & 1];
        CILREG_TRY(rof_launch_step(cur, nxt, f, nullptr, lam, tau, d, ctl, 0, nullptr, s));
        cur = nxt;
    }

    // reverse sweep from W = ybar
    CILREG_CUDA(cudaMemcpyAsync(wb[0], ybar, nb, cudaMemcpyDeviceToDevice, s));
    int wi = 0;
    for (int g = nseg - 1; g >= 0; g--) {
        const int k0 = g * ckpt, k1 = (k0 + ckpt < L) ? k0 + ckpt : L;
        const float* start = (g == 0) ? f : ck[g];
        auto state = [&](int k) -> const float* { return (k == k0) ? start : seg[k - k0]; };
        for (int k = k0; k + 1 < k1; k++)
            CILREG_TRY(rof_launch_step(state(k), seg[k + 1 - k0], f, nullptr, lam, tau, d, ctl, 0, nullptr, s));
        for (int k = k1 - 1; k >= k0; k--) {
            RofAdjArgs a;
            a.u = state(k);
            a.w = wb[wi];
            for (int c = 0; c < 3; c++) {
                a.e[c] = E[c];
                a.fq[c] = Fq[c];
            }
            a.ubar = wb[wi ^ 1];
            a.fbar = fbar;
            a.lam = lam;
            a.tau = tau;
            if (three) {
                k_rof_adj_coef<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_rof_adj_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc);
                k_rof_adj_gather<true><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
            } else {
                k_rof_adj_coef<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz, part);
                k_rof_adj_accumulate<<<1, 1024, 0, s>>>(part, num_blocks(LA), acc);
                k_rof_adj_gather<false><<<LA.grid, LA.block, 0, s>>>(a, d, LA.kz);
            }
            CILREG_CUDA(cudaGetLastError());
            note_launch(3);
            wi ^= 1;
        }
    }
    // U_0 = f: its adjoint joins fbar
    k_rof_adj_add<<<grid1(n), 256, 0, s>>>(fbar, wb[wi], n);
    CILREG_CUDA(cudaGetLastError());
    note_launch();
    double h = 0.0;
    CILREG_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (lambar) *lambar = (double)tau * h;
    return OK;
}

}  // namespace cilreg

using namespace cilreg;

extern "C" int cilreg_rof_tv_vjp_dev(const float* d_in, const float* d_ybar, float* d_inbar, double* lambar,
                                     float lambdaPar, int iters, float tau, int checkpoint, int dimX, int dimY,
                                     int dimZ, void* stream) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    if (!d_in || !d_ybar || !d_inbar) return fail(ERR_ARG, __FILE__, __LINE__, "null device pointer");
    return rof_vjp_run(d_in, d_ybar, lambdaPar, iters, tau, checkpoint, make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ),
                       (cudaStream_t)stream, d_inbar, lambar);
}
