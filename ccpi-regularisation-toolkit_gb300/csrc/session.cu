// Prox sessions: a regulariser whose state stays on the device across the
// outer iterations of a proximal-splitting solver, and the FISTA outer loop
// of the denoising problem  min_x 1/2 ||x - f||^2 + R(x)  built on it.
//
// The reference discards every variable at the end of each call
// (TV_FGP_GPU_core.cu:586-598, TV_SB_GPU_core.cu:519-533), so an outer solver
// pays a cold start per prox.  A session keeps
//   FGP-TV  the dual iterates P (three ring buffers)
//   SB-TV   the split and Bregman variables D, B
//   ROF-TV, NDF  the previous prox output (the starting iterate of the next)
// plus the solver's x, y, z buffers, in one device allocation whose size
// cilreg_prox_session_bytes reports in advance (for admission control).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <new>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"
#include "nvtx.cuh"

namespace cilreg {
namespace {

enum { ALG_ROF = 0, ALG_FGP = 1, ALG_SB = 2, ALG_NDF = 3 };

size_t arr_bytes(const Dims& d) { return ((sizeof(float) * (size_t)d.n) + 255) & ~(size_t)255; }

// number of volume-sized arrays a session holds, and the transient scratch the
// prox call itself takes from the pool (for the admission estimate)
int held_arrays(int alg, bool three) {
    const int nc = three ? 3 : 2;
    switch (alg) {
        case ALG_FGP: return 3 * nc + 4;  // ring + x, y, z, xn
        case ALG_SB: return 2 * nc + 4;   // D, B + x, y, z, xn
        default: return 5;                // previous output + x, y, z, xn
    }
}
int transient_arrays(int alg, bool three) {
    if (alg == ALG_FGP) return 1;
    if (alg == ALG_SB) return 1 + (three ? 3 : 2);  // U ping-pong + B ping-pong
    return 2;
}

__global__ void k_grad_step(float* __restrict__ z, const float* __restrict__ y, const float* __restrict__ f,
                            float step, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) z[i] = y[i] - step * (y[i] - f[i]);
}

__global__ void k_momentum(float* __restrict__ y, const float* __restrict__ xn, const float* __restrict__ x,
                           float beta, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) y[i] = xn[i] + beta * (xn[i] - x[i]);
}

// ADMM (scaled form) on min_x 1/2 ||w^(1/2)(x - f)||^2 + R(x) with the
// splitting x = z:  x = (w f + rho (z - u)) / (w + rho),  v = x + u  (the
// prox argument; z = prox(v) follows),  then  u = u + x - z.
__global__ void k_admm_xv(float* __restrict__ x, float* __restrict__ v, const float* __restrict__ z,
                          const float* __restrict__ u, const float* __restrict__ f, const float* __restrict__ w,
                          float rho, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        const float wi = w ? w[i] : 1.0f;
        const float xi = __fdiv_rn(__fadd_rn(__fmul_rn(wi, f[i]), __fmul_rn(rho, __fsub_rn(z[i], u[i]))),
                                   __fadd_rn(wi, rho));
        x[i] = xi;
        v[i] = __fadd_rn(xi, u[i]);
    }
}

__global__ void k_admm_u(float* __restrict__ u, const float* __restrict__ x, const float* __restrict__ z,
                         long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) u[i] = __fsub_rn(__fadd_rn(u[i], x[i]), z[i]);
}

// PDHG (Chambolle-Pock, K = I) on the same problem with the regulariser as
// the dual term:  y+ = prox_{sigma R*}(y + sigma xbar) = sigma (q - prox_{R/sigma}(q))
// with q = y / sigma + xbar;  x+ = (x - tau y+ + tau w f) / (1 + tau w);
// xbar = 2 x+ - x.  q is formed in place over xbar.
__global__ void k_pdhg_q(float* __restrict__ q, const float* __restrict__ y, float inv_sigma, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) q[i] = __fadd_rn(__fmul_rn(y[i], inv_sigma), q[i]);
}

__global__ void k_pdhg_primal(float* __restrict__ x, float* __restrict__ y, float* __restrict__ qbar,
                              const float* __restrict__ p, const float* __restrict__ f, const float* __restrict__ w,
                              float tau, float sigma, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        const float wi = w ? w[i] : 1.0f;
        const float yi = __fmul_rn(sigma, __fsub_rn(qbar[i], p[i]));
        const float tw = __fmul_rn(tau, wi);
        const float xo = x[i];
        const float xn = __fdiv_rn(__fadd_rn(__fsub_rn(xo, __fmul_rn(tau, yi)), __fmul_rn(tw, f[i])),
                                   __fadd_rn(1.0f, tw));
        y[i] = yi;
        x[i] = xn;
        qbar[i] = __fsub_rn(__fmul_rn(2.0f, xn), xo);
    }
}

dim3 ew_grid(long long n) {
    long long b = (n + 255) / 256;
    if (b > 152LL * 8) b = 152LL * 8;
    return dim3((unsigned)(b < 1 ? 1 : b));
}

}  // namespace
}  // namespace cilreg

using namespace cilreg;

struct cilreg_session {
    int alg;
    Dims d;
    float prm[4];
    void* block;
    size_t bytes;
    float *x, *y, *z, *xn, *uprev;
    bool has_prev;
    FgpWarm fgp;
    SbWarm sb;
    const volatile int* cancel;  // host flag: nonzero ends an outer loop after its current step
};

namespace {

int session_prox(cilreg_session* S, const float* in, float* out, int iters, float epsil, float* info,
                 cudaStream_t s) {
    const Dims& d = S->d;
    int rc = OK;
    switch (S->alg) {
        case ALG_FGP:
            rc = fgp_run(in, out, S->prm[0], iters, epsil, (int)S->prm[1], (int)S->prm[2], d, s, info, &S->fgp);
            break;
        case ALG_SB:
            rc = sb_run(in, out, S->prm[0], iters, epsil, (int)S->prm[1], d, s, info, &S->sb);
            break;
        case ALG_ROF:
            rc = rof_run(in, out, nullptr, S->prm[0], iters, S->prm[1], epsil, d, s, info,
                         S->has_prev ? S->uprev : nullptr);
            break;
        case ALG_NDF:
            rc = ndf_run(in, out, S->prm[0], S->prm[1], iters, S->prm[2], (int)S->prm[3], epsil, d, s, info,
                         S->has_prev ? S->uprev : nullptr);
            break;
        default:
            return fail(ERR_ARG, __FILE__, __LINE__, "unknown session algorithm %d", S->alg);
    }
    if (rc != OK) return rc;
    if (S->alg == ALG_ROF || S->alg == ALG_NDF) {
        CILREG_CUDA(cudaMemcpyAsync(S->uprev, out, sizeof(float) * (size_t)d.n, cudaMemcpyDeviceToDevice, s));
        S->has_prev = true;
    }
    return OK;
}

// between two outer steps: with a cancel flag registered, wait for the step
// (so that cancelling takes effect within one step) and report a raised flag
int outer_boundary(cilreg_session* S, cudaStream_t s) {
    if (!S->cancel) return OK;
    CILREG_CUDA(cudaStreamSynchronize(s));
    if (*S->cancel) return fail(ERR_CANCELLED, __FILE__, __LINE__, "cancelled");
    return OK;
}

}  // namespace

extern "C" {

long long cilreg_prox_session_bytes(int alg, int dimX, int dimY, int dimZ) {
    if (check_dims(dimX, dimY, dimZ) != 0 || alg < 0 || alg > 3) return -1;
    const Dims d = make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ);
    return (long long)(arr_bytes(d) * (size_t)(held_arrays(alg, d.nz > 1) + transient_arrays(alg, d.nz > 1))) + (1 << 20);
}

int cilreg_prox_session_create(cilreg_session** out, int alg, const float* params, int nparams, int dimX, int dimY,
                               int dimZ, void* stream) {
    if (!out) return fail(ERR_ARG, __FILE__, __LINE__, "null session pointer");
    *out = nullptr;
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    static const int need[4] = {2, 3, 2, 4};
    if (alg < 0 || alg > 3) return fail(ERR_ARG, __FILE__, __LINE__, "unknown algorithm %d (0 ROF, 1 FGP, 2 SB, 3 NDF)", alg);
    if (!params || nparams < need[alg])
        return fail(ERR_ARG, __FILE__, __LINE__, "algorithm %d needs %d parameters", alg, need[alg]);
    cilreg_session* S = new (std::nothrow) cilreg_session();
    if (!S) return fail(ERR_OOM, __FILE__, __LINE__, "host allocation failed");
    S->cancel = nullptr;
    if (take_injected_failure()) {
        delete S;
        return fail(ERR_OOM, __FILE__, __LINE__, "session allocation failed: injected failure");
    }
    S->alg = alg;
    S->d = make_dims(dimX, dimY, dimZ < 1 ? 1 : dimZ);
    for (int i = 0; i < 4; i++) S->prm[i] = (i < nparams) ? params[i] : 0.0f;
    const bool three = S->d.nz > 1;
    const int nc = three ? 3 : 2;
    const size_t ab = arr_bytes(S->d);
    const int narr = held_arrays(alg, three);
    S->bytes = ab * (size_t)narr;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMallocAsync(&S->block, S->bytes, s);
    if (e != cudaSuccess) {
        delete S;
        return fail(e == cudaErrorMemoryAllocation ? ERR_OOM : ERR_CUDA, __FILE__, __LINE__,
                    "session allocation of %zu bytes failed: %s", (size_t)(ab * narr), cudaGetErrorString(e));
    }
    char* p = (char*)S->block;
    auto take = [&]() {
        float* r = (float*)p;
        p += ab;
        return r;
    };
    S->x = take();
    S->y = take();
    S->z = take();
    S->xn = take();
    S->uprev = nullptr;
    S->has_prev = false;
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) S->fgp.ring[r][c] = nullptr;
    for (int c = 0; c < 3; c++) S->sb.dd[c] = S->sb.bb[c] = nullptr;
    S->fgp.base = 0;
    if (alg == ALG_FGP) {
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < nc; c++) S->fgp.ring[r][c] = take();
    } else if (alg == ALG_SB) {
        for (int c = 0; c < nc; c++) {
            S->sb.dd[c] = take();
            S->sb.bb[c] = take();
        }
    } else {
        S->uprev = take();
    }
    // cold state: zero duals / split variables
    e = cudaMemsetAsync(S->block, 0, S->bytes, s);
    if (e != cudaSuccess) {
        cudaFreeAsync(S->block, s);
        delete S;
        return fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(e));
    }
    *out = S;
    return OK;
}

int cilreg_prox_session_prox(cilreg_session* S, const float* d_in, float* d_out, int iters, float epsil,
                             float* infovector, void* stream) {
    CILREG_RANGE("cilreg prox");
    if (!S || !d_in || !d_out || d_in == d_out) return fail(ERR_ARG, __FILE__, __LINE__, "bad session call");
    return session_prox(S, d_in, d_out, iters, epsil, infovector, (cudaStream_t)stream);
}

int cilreg_prox_session_fista(cilreg_session* S, const float* d_f, float* d_x, int outer, int inner, float step,
                              void* stream) {
    CILREG_RANGE("cilreg FISTA");
    if (!S || !d_f || !d_x) return fail(ERR_ARG, __FILE__, __LINE__, "bad session call");
    if (outer < 0 || inner < 0) return fail(ERR_ARG, __FILE__, __LINE__, "negative iteration count");
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = S->d.n;
    const size_t nb = sizeof(float) * (size_t)n;
    CILREG_CUDA(cudaMemcpyAsync(S->x, d_f, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(S->y, d_f, nb, cudaMemcpyDeviceToDevice, s));
    float t = 1.0f;
    for (int k = 0; k < outer; k++) {
        CILREG_TRY(outer_boundary(S, s));
        k_grad_step<<<ew_grid(n), 256, 0, s>>>(S->z, S->y, d_f, step, n);  // gradient of 1/2 ||y - f||^2
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        CILREG_TRY(session_prox(S, S->z, S->xn, inner, 0.0f, nullptr, s));
        const float tn = (1.0f + sqrtf(1.0f + 4.0f * t * t)) * 0.5f;
        k_momentum<<<ew_grid(n), 256, 0, s>>>(S->y, S->xn, S->x, (t - 1.0f) / tn, n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        float* tmp = S->x;
        S->x = S->xn;
        S->xn = tmp;
        t = tn;
    }
    CILREG_CUDA(cudaMemcpyAsync(d_x, S->x, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}

int cilreg_prox_session_admm(cilreg_session* S, const float* d_f, const float* d_w, float* d_x, int outer, int inner,
                             float rho, void* stream) {
    CILREG_RANGE("cilreg ADMM");
    if (!S || !d_f || !d_x) return fail(ERR_ARG, __FILE__, __LINE__, "bad session call");
    if (outer < 0 || inner < 0) return fail(ERR_ARG, __FILE__, __LINE__, "negative iteration count");
    if (!(rho > 0.0f)) return fail(ERR_ARG, __FILE__, __LINE__, "rho must be positive");
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = S->d.n;
    const size_t nb = sizeof(float) * (size_t)n;
    // x in S->x, u in S->y, the prox argument v in S->z, z in S->xn
    CILREG_CUDA(cudaMemcpyAsync(S->xn, d_f, nb, cudaMemcpyDeviceToDevice, s));  // z = f
    CILREG_CUDA(cudaMemsetAsync(S->y, 0, nb, s));                                  // u = 0
    for (int k = 0; k < outer; k++) {
        CILREG_TRY(outer_boundary(S, s));
        k_admm_xv<<<ew_grid(n), 256, 0, s>>>(S->x, S->z, S->xn, S->y, d_f, d_w, rho, n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        CILREG_TRY(session_prox(S, S->z, S->xn, inner, 0.0f, nullptr, s));
        k_admm_u<<<ew_grid(n), 256, 0, s>>>(S->y, S->x, S->xn, n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
    }
    CILREG_CUDA(cudaMemcpyAsync(d_x, S->xn, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}

int cilreg_prox_session_pdhg(cilreg_session* S, const float* d_f, const float* d_w, float* d_x, int outer, int inner,
                             float tau, float sigma, void* stream) {
    CILREG_RANGE("cilreg PDHG");
    if (!S || !d_f || !d_x) return fail(ERR_ARG, __FILE__, __LINE__, "bad session call");
    if (outer < 0 || inner < 0) return fail(ERR_ARG, __FILE__, __LINE__, "negative iteration count");
    if (!(tau > 0.0f) || !(sigma > 0.0f)) return fail(ERR_ARG, __FILE__, __LINE__, "tau and sigma must be positive");
    cudaStream_t s = (cudaStream_t)stream;
    const long long n = S->d.n;
    const size_t nb = sizeof(float) * (size_t)n;
    // x in S->x, the dual y in S->y, xbar (then q in place) in S->z, prox(q) in S->xn
    CILREG_CUDA(cudaMemcpyAsync(S->x, d_f, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaMemcpyAsync(S->z, d_f, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaMemsetAsync(S->y, 0, nb, s));
    const float inv_sigma = 1.0f / sigma;
    for (int k = 0; k < outer; k++) {
        CILREG_TRY(outer_boundary(S, s));
        k_pdhg_q<<<ew_grid(n), 256, 0, s>>>(S->z, S->y, inv_sigma, n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
        CILREG_TRY(session_prox(S, S->z, S->xn, inner, 0.0f, nullptr, s));
        k_pdhg_primal<<<ew_grid(n), 256, 0, s>>>(S->x, S->y, S->z, S->xn, d_f, d_w, tau, sigma, n);
        CILREG_CUDA(cudaGetLastError());
        note_launch();
    }
    CILREG_CUDA(cudaMemcpyAsync(d_x, S->x, nb, cudaMemcpyDeviceToDevice, s));
    CILREG_CUDA(cudaStreamSynchronize(s));
    return OK;
}

int cilreg_prox_session_set_cancel(cilreg_session* S, const volatile int* flag) {
    if (!S) return fail(ERR_ARG, __FILE__, __LINE__, "null session");
    S->cancel = flag;
    return OK;
}

int cilreg_debug_fail_allocations(int n) {
    inject_allocation_failures(n);
    return OK;
}

int cilreg_prox_session_destroy(cilreg_session* S, void* stream) {
    if (!S) return OK;
    cudaError_t e = cudaFreeAsync(S->block, (cudaStream_t)stream);
    delete S;
    if (e != cudaSuccess) return fail(ERR_CUDA, __FILE__, __LINE__, "%s", cudaGetErrorString(e));
    return OK;
}

}  // extern "C"
