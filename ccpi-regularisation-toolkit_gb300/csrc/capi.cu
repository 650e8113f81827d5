// The C ABI: drop-in entry points with the reference's argument lists.
//
//  * *_GPU_main    host pointers in/out, explicit gpu_device, int status
//                  (src/Core/regularisers_GPU/*.h, headers/*.h)
//  * *_CPU_main    the C-OMP argument lists (src/Core/regularisers_CPU/*_core.h);
//                  in this library they execute on the GPU selected by
//                  CILREG_GPU_DEVICE (default 0) and return 0 or a negative status
//  * cilreg_*_dev  device pointers and a caller stream (cudaStream_t as void*)
//
// Every entry point validates its arguments, returns a status instead of
// printing and continuing, and is safe to call from several host threads
// (each thread gets its own stream; scratch is stream-ordered).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/mman.h>
#include <unistd.h>

#include <chrono>
#include <thread>

#include "../../include/cilreg_gb300.h"
#include "drivers.cuh"

using namespace cilreg;

namespace cilreg {

int check_dims(int nx, int ny, int nz) {
    if (nx < 1 || ny < 1 || nz < 0)
        return fail(ERR_ARG, __FILE__, __LINE__, "invalid dimensions (%d, %d, %d)", nx, ny, nz);
    return OK;
}

}  // namespace cilreg

namespace {

Dims dims_of(int nx, int ny, int nz) { return make_dims(nx, ny, nz < 1 ? 1 : nz); }

int default_device() {
    const char* e = getenv("CILREG_GPU_DEVICE");
    return e ? atoi(e) : 0;
}

// Map every page of the caller's output buffer for writing, without changing
// its contents (MADV_POPULATE_WRITE).  A freshly allocated host array (numpy
// zeros_like, calloc) is backed by pages that only fault in when first
// written; the download would otherwise take those faults itself, tens of
// milliseconds per 512 MiB.  Runs on a helper thread while the GPU iterates.
void populate_for_write(void* p, size_t bytes) {
#ifdef MADV_POPULATE_WRITE
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    const uintptr_t a = (uintptr_t)p & ~(uintptr_t)(page - 1);
    const uintptr_t e = ((uintptr_t)p + bytes + page - 1) & ~(uintptr_t)(page - 1);
    madvise((void*)a, e - a, MADV_POPULATE_WRITE);  // best effort: an error leaves the faults to the copy
#else
    (void)p;
    (void)bytes;
#endif
}

// Host-pointer wrapper: upload input (and the output buffer when `upload_out`),
// run `body(d_in, d_out, stream)`, download the output.  Outputs of 16 MiB or
// more are populated for writing on a helper thread meanwhile.
template <class Body>
int host_call(const float* in, float* out, int dev, const Dims& d, bool upload_out, Body body) {
    if (!in || !out) return fail(ERR_ARG, __FILE__, __LINE__, "null Input/Output pointer");
    CILREG_TRY(use_device(dev));
    cudaStream_t s = thread_stream(dev);
    int rc;
    {
        Scratch io(s);
        float* d_in = io.floats(d.n);
        float* d_out = io.floats(d.n);
        if (!d_in || !d_out) return io.status();
        const size_t bytes = sizeof(float) * (size_t)d.n;
        // CILREG_HOST_TIMING=1 prints the phases of the call to stderr (diagnostic)
        const bool timing = getenv("CILREG_HOST_TIMING") != nullptr;
        const auto t0 = std::chrono::steady_clock::now();
        auto ms_since = [&](std::chrono::steady_clock::time_point a) {
            return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - a).count();
        };
        CILREG_CUDA(cudaMemcpyAsync(d_in, in, bytes, cudaMemcpyHostToDevice, s));
        if (upload_out) CILREG_CUDA(cudaMemcpyAsync(d_out, out, bytes, cudaMemcpyHostToDevice, s));
        if (timing) CILREG_CUDA(cudaStreamSynchronize(s));
        const double t_up = timing ? ms_since(t0) : 0.0;
        std::thread pre;
        double t_pop = 0.0;
        if (bytes >= (16u << 20))
            pre = std::thread([&] {
                const auto p0 = std::chrono::steady_clock::now();
                populate_for_write((void*)out, bytes);
                t_pop = ms_since(p0);
            });
        const auto t1 = std::chrono::steady_clock::now();
        rc = body(d_in, d_out, s);
        if (timing) cudaStreamSynchronize(s);
        const double t_body = timing ? ms_since(t1) : 0.0;
        if (pre.joinable()) pre.join();
        const double t_join = timing ? ms_since(t1) - t_body : 0.0;
        if (rc == 0) {
            const auto t2 = std::chrono::steady_clock::now();
            CILREG_CUDA(cudaMemcpyAsync(out, d_out, bytes, cudaMemcpyDeviceToHost, s));
            CILREG_CUDA(cudaStreamSynchronize(s));
            if (timing)
                fprintf(stderr, "cilreg host call: upload %.2f ms, run %.2f ms, populate %.2f ms (waited %.2f), "
                        "download %.2f ms, total %.2f ms\n", t_up, t_body, t_pop, t_join, ms_since(t2), ms_since(t0));
        }
    }
    return rc;
}

int dev_prologue(const float* in, const float* out, int nx, int ny, int nz) {
    CILREG_TRY(check_dims(nx, ny, nz));
    if (!in || !out) return fail(ERR_ARG, __FILE__, __LINE__, "null device pointer");
    if (in == out) return fail(ERR_ARG, __FILE__, __LINE__, "input and output must be distinct buffers");
    return OK;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// library information
const char* cilreg_last_error(void) { return last_error(); }
const char* cilreg_version(void) { return "cilreg-gb300 1.0 (sm_103a)"; }
long long cilreg_launch_count(void) { return launch_count(); }
int cilreg_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

int cilreg_release_cached(int gpu_device) { return release_cached(gpu_device); }

// ---------------------------------------------------------------------------
// device-pointer API
int cilreg_rof_tv_dev(const float* d_in, float* d_out, float* infovector, const float* d_lambda, float lambdaPar,
                      int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return rof_run(d_in, d_out, d_lambda, lambdaPar, iters, tau, epsil, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

int cilreg_fgp_tv_dev(const float* d_in, float* d_out, float* infovector, float lambdaPar, int iters, float epsil,
                      int methodTV, int nonneg, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return fgp_run(d_in, d_out, lambdaPar, iters, epsil, methodTV, nonneg, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

int cilreg_pd_tv_dev(const float* d_in, float* d_out, float* infovector, float lambdaPar, int iters, float epsil,
                     float lipschitz_const, int methodTV, int nonneg, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return pd_run(d_in, d_out, lambdaPar, iters, epsil, lipschitz_const, methodTV, nonneg, dims_of(dimX, dimY, dimZ),
                  (cudaStream_t)stream, infovector);
}

int cilreg_sb_tv_dev(const float* d_in, float* d_out, float* infovector, float mu, int iters, float epsil,
                     int methodTV, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return sb_run(d_in, d_out, mu, iters, epsil, methodTV, dims_of(dimX, dimY, dimZ), (cudaStream_t)stream,
                  infovector);
}

int cilreg_tgv_dev(const float* d_in, float* d_out, float* infovector, float lambdaPar, float alpha1, float alpha0,
                   int iters, float L2, float epsil, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return tgv_run(d_in, d_out, lambdaPar, alpha1, alpha0, iters, L2, epsil, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

int cilreg_ndf_dev(const float* d_in, float* d_out, float* infovector, float lambdaPar, float sigmaPar, int iters,
                   float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return ndf_run(d_in, d_out, lambdaPar, sigmaPar, iters, tau, penaltytype, epsil, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

int cilreg_diff4th_dev(const float* d_in, float* d_out, float* infovector, float lambdaPar, float sigmaPar,
                       int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return diff4th_run(d_in, d_out, lambdaPar, sigmaPar, iters, tau, epsil, dims_of(dimX, dimY, dimZ),
                       (cudaStream_t)stream, infovector);
}

int cilreg_llt_rof_dev(const float* d_in, float* d_out, float* infovector, float lambdaROF, float lambdaLLT,
                       int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    return llt_run(d_in, d_out, lambdaROF, lambdaLLT, iters, tau, epsil, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

int cilreg_dtv_fgp_dev(const float* d_in, const float* d_ref, float* d_out, float* infovector, float lambdaPar,
                       int iters, float epsil, float eta, int methodTV, int nonneg, int dimX, int dimY, int dimZ,
                       void* stream) {
    CILREG_TRY(dev_prologue(d_in, d_out, dimX, dimY, dimZ));
    if (!d_ref) return fail(ERR_ARG, __FILE__, __LINE__, "null reference image");
    return dtv_run(d_in, d_ref, d_out, lambdaPar, iters, epsil, eta, methodTV, nonneg, dims_of(dimX, dimY, dimZ),
                   (cudaStream_t)stream, infovector);
}

// ---------------------------------------------------------------------------
// *_GPU_main: the reference GPU ABI (host pointers)
int TV_ROF_GPU_main(float* Input, float* Output, float* infovector, float lambdaPar, int iter, float tau, float epsil,
                    int gpu_device, int N, int M, int Z) {
    CILREG_TRY(check_dims(N, M, Z));
    const Dims d = dims_of(N, M, Z);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return rof_run(di, dout, nullptr, lambdaPar, iter, tau, epsil, d, s, infovector);
    });
}

int TV_FGP_GPU_main(float* Input, float* Output, float* infovector, float lambdaPar, int iter, float epsil,
                    int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    const Dims d = dims_of(dimX, dimY, dimZ);
    // U_prev of iteration 0: the C-OMP path takes the caller's Output
    // (FGP_TV_core.c:66,123, zeros from the Python layer); the reference GPU
    // path copies its uninitialised device U instead (TV_FGP_GPU_core.cu:377,
    // 516).  Here it is zero on the device, so the caller's Output is not
    // uploaded (it is, unchanged, when no iteration runs).
    return host_call(Input, Output, gpu_device, d, iter <= 0, [&](const float* di, float* dout, cudaStream_t s) {
        if (epsil != 0.0f && iter > 0) CILREG_CUDA(cudaMemsetAsync(dout, 0, sizeof(float) * d.n, s));
        return fgp_run(di, dout, lambdaPar, iter, epsil, methodTV, nonneg, d, s, infovector);
    });
}

int TV_PD_GPU_main(float* Input, float* Output, float* infovector, float lambdaPar, int iter, float epsil,
                   float lipschitz_const, int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    const Dims d = dims_of(dimX, dimY, dimZ);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return pd_run(di, dout, lambdaPar, iter, epsil, lipschitz_const, methodTV, nonneg, d, s, infovector);
    });
}

int TV_SB_GPU_main(float* Input, float* Output, float* infovector, float mu, int iter, float epsil, int methodTV,
                   int gpu_device, int dimX, int dimY, int dimZ) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    const Dims d = dims_of(dimX, dimY, dimZ);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return sb_run(di, dout, mu, iter, epsil, methodTV, d, s, infovector);
    });
}

int TGV_GPU_main(float* U0, float* U, float* infovector, float lambda, float alpha1, float alpha0, int iterationsNumb,
                 float L2, float epsil, int gpu_device, int dimX, int dimY, int dimZ) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    const Dims d = dims_of(dimX, dimY, dimZ);
    return host_call(U0, U, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return tgv_run(di, dout, lambda, alpha1, alpha0, iterationsNumb, L2, epsil, d, s, infovector);
    });
}

int NonlDiff_GPU_main(float* Input, float* Output, float* infovector, float lambdaPar, float sigmaPar,
                      int iterationsNumb, float tau, int penaltytype, float epsil, int gpu_device, int N, int M,
                      int Z) {
    CILREG_TRY(check_dims(N, M, Z));
    const Dims d = dims_of(N, M, Z);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return ndf_run(di, dout, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype, epsil, d, s, infovector);
    });
}

int Diffus4th_GPU_main(float* Input, float* Output, float* infovector, float lambdaPar, float sigmaPar,
                       int iterationsNumb, float tau, float epsil, int gpu_device, int N, int M, int Z) {
    CILREG_TRY(check_dims(N, M, Z));
    const Dims d = dims_of(N, M, Z);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return diff4th_run(di, dout, lambdaPar, sigmaPar, iterationsNumb, tau, epsil, d, s, infovector);
    });
}

int LLT_ROF_GPU_main(float* Input, float* Output, float* infovector, float lambdaROF, float lambdaLLT,
                     int iterationsNumb, float tau, float epsil, int gpu_device, int N, int M, int Z) {
    CILREG_TRY(check_dims(N, M, Z));
    const Dims d = dims_of(N, M, Z);
    return host_call(Input, Output, gpu_device, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        return llt_run(di, dout, lambdaROF, lambdaLLT, iterationsNumb, tau, epsil, d, s, infovector);
    });
}

int dTV_FGP_GPU_main(float* Input, float* InputRef, float* Output, float* infovector, float lambdaPar, int iter,
                     float epsil, float eta, int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ) {
    CILREG_TRY(check_dims(dimX, dimY, dimZ));
    if (!InputRef) return fail(ERR_ARG, __FILE__, __LINE__, "null InputRef pointer");
    const Dims d = dims_of(dimX, dimY, dimZ);
    // as FGP: U_prev of iteration 0 is zero on the device (dTV_FGP_GPU_core.cu
    // leaves it uninitialised; the C-OMP path takes the caller's Output)
    return host_call(Input, Output, gpu_device, d, iter <= 0,
                     [&](const float* di, float* dout, cudaStream_t s) {
                         if (epsil != 0.0f && iter > 0)
                             CILREG_CUDA(cudaMemsetAsync(dout, 0, sizeof(float) * d.n, s));
                         Scratch sc(s);
                         float* dr = sc.floats(d.n);
                         if (!dr) return sc.status();
                         CILREG_CUDA(cudaMemcpyAsync(dr, InputRef, sizeof(float) * d.n, cudaMemcpyHostToDevice, s));
                         return dtv_run(di, dr, dout, lambdaPar, iter, epsil, eta, methodTV, nonneg, d, s,
                                        infovector);
                     });
}

// ---------------------------------------------------------------------------
// *_CPU_main: the reference C-OMP ABI, executed on the GPU
float TV_ROF_CPU_main(float* Input, float* Output, float* infovector, float* lambdaPar, int lambda_is_arr,
                      int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ) {
    if (check_dims(dimX, dimY, dimZ) != 0) return (float)ERR_ARG;
    if (!lambdaPar) return (float)fail(ERR_ARG, __FILE__, __LINE__, "null lambdaPar");
    const Dims d = dims_of(dimX, dimY, dimZ);
    const int dev = default_device();
    return (float)host_call(Input, Output, dev, d, false, [&](const float* di, float* dout, cudaStream_t s) {
        if (!lambda_is_arr) return rof_run(di, dout, nullptr, *lambdaPar, iterationsNumb, tau, epsil, d, s, infovector);
        Scratch sc(s);
        float* dl = sc.floats(d.n);
        if (!dl) return sc.status();
        CILREG_CUDA(cudaMemcpyAsync(dl, lambdaPar, sizeof(float) * d.n, cudaMemcpyHostToDevice, s));
        return rof_run(di, dout, dl, 0.0f, iterationsNumb, tau, epsil, d, s, infovector);
    });
}

float TV_FGP_CPU_main(float* Input, float* Output, float* infovector, float lambdaPar, int iterationsNumb, float epsil,
                      int methodTV, int nonneg, int dimX, int dimY, int dimZ) {
    return (float)TV_FGP_GPU_main(Input, Output, infovector, lambdaPar, iterationsNumb, epsil, methodTV, nonneg,
                                  default_device(), dimX, dimY, dimZ);
}

float PDTV_CPU_main(float* Input, float* U, float* infovector, float lambdaPar, int iterationsNumb, float epsil,
                    float lipschitz_const, int methodTV, int nonneg, int dimX, int dimY, int dimZ) {
    return (float)TV_PD_GPU_main(Input, U, infovector, lambdaPar, iterationsNumb, epsil, lipschitz_const, methodTV,
                                 nonneg, default_device(), dimX, dimY, dimZ);
}

float SB_TV_CPU_main(float* Input, float* Output, float* infovector, float mu, int iter, float epsil, int methodTV,
                     int dimX, int dimY, int dimZ) {
    return (float)TV_SB_GPU_main(Input, Output, infovector, mu, iter, epsil, methodTV, default_device(), dimX, dimY,
                                 dimZ);
}

float TGV_main(float* U0, float* U, float* infovector, float lambda, float alpha1, float alpha0, int iter, float L2,
               float epsil, int dimX, int dimY, int dimZ) {
    return (float)TGV_GPU_main(U0, U, infovector, lambda, alpha1, alpha0, iter, L2, epsil, default_device(), dimX,
                               dimY, dimZ);
}

float Diffusion_CPU_main(float* Input, float* Output, float* infovector, float lambdaPar, float sigmaPar,
                         int iterationsNumb, float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ) {
    return (float)NonlDiff_GPU_main(Input, Output, infovector, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype,
                                    epsil, default_device(), dimX, dimY, dimZ);
}

float Diffus4th_CPU_main(float* Input, float* Output, float* infovector, float lambdaPar, float sigmaPar,
                         int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ) {
    return (float)Diffus4th_GPU_main(Input, Output, infovector, lambdaPar, sigmaPar, iterationsNumb, tau, epsil,
                                     default_device(), dimX, dimY, dimZ);
}


float LLT_ROF_CPU_main(float* Input, float* Output, float* infovector, float lambdaROF, float lambdaLLT,
                       int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ) {
    return (float)LLT_ROF_GPU_main(Input, Output, infovector, lambdaROF, lambdaLLT, iterationsNumb, tau, epsil,
                                   default_device(), dimX, dimY, dimZ);
}

float dTV_FGP_CPU_main(float* Input, float* InputRef, float* Output, float* infovector, float lambdaPar,
                       int iterationsNumb, float epsil, float eta, int methodTV, int nonneg, int dimX, int dimY,
                       int dimZ) {
    return (float)dTV_FGP_GPU_main(Input, InputRef, Output, infovector, lambdaPar, iterationsNumb, epsil, eta,
                                   methodTV, nonneg, default_device(), dimX, dimY, dimZ);
}

}  // extern "C"
