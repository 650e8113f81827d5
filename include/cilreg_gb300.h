/*
 * cilreg_gb300.h — C ABI of the GB300 (sm_103a) proximal regularisers.
 *
 * Drop-in for the CCPi Regularisation Toolkit's shared libraries:
 *   libcilregcuda.so  holds every entry point below (the *_GPU_main and
 *                     *_CPU_main families and the cilreg_* API);
 *   libcilreg.so      exports the same entry points, each forwarding to
 *                     libcilregcuda.so in its directory, so that a process
 *                     binding both names holds one copy of the GPU library.
 *
 * Arrays are C-ordered float32 with dimX the fastest axis: linear index
 * (dimX*dimY)*k + dimX*j + i.  A 2D image has dimZ == 1 (dimZ == 0 is read as 1).
 *
 * infovector (host pointer to 2 floats, may be NULL) receives
 *   [iterations run (the break index when the stopping rule fired), last relative change].
 * Stopping rule: when epsil != 0, every 5th iteration re = ||U - U_prev|| / ||U||,
 * a counter increments when re < epsil and the run stops once it exceeds 3.
 *
 * Return values: 0 on success, negative on failure
 *   -1 CUDA error, -2 invalid argument, -3 no CUDA device, -4 out of device memory,
 *   -5 cancelled (prox-session outer loops only);
 * the message is available from cilreg_last_error() (per host thread) and is
 * also printed to stderr, as the reference does (regularisers_GPU/shared.h:15-38).
 * All entry points may be called concurrently from several host threads.
 *
 * Deliberate differences from the reference are listed with each function.
 */
#ifndef CILREG_GB300_H
#define CILREG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Reference GPU ABI (host pointers in/out; the call copies to and from the
 * device and returns when Output is filled).
 * ------------------------------------------------------------------------- */

/* replaces TV_ROF_GPU_main, src/Core/regularisers_GPU/headers/TV_ROF_GPU_core.h:6 */
int TV_ROF_GPU_main(float *Input, float *Output, float *infovector, float lambdaPar, int iter, float tau,
                    float epsil, int gpu_device, int N, int M, int Z);

/* replaces TV_FGP_GPU_main, src/Core/regularisers_GPU/TV_FGP_GPU_core.h:7.
 * U_prev of iteration 0 is zero (the reference GPU path leaves it
 * uninitialised; TV_FGP_CPU_main takes Output's initial content, as the CPU
 * reference does); Output is only written. */
int TV_FGP_GPU_main(float *Input, float *Output, float *infovector, float lambdaPar, int iter, float epsil,
                    int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ);

/* replaces TV_PD_GPU_main, src/Core/regularisers_GPU/headers/TV_PD_GPU_core.h:7.
 * infovector needs 2 floats (the reference's Python passes an image-sized one). */
int TV_PD_GPU_main(float *Input, float *Output, float *infovector, float lambdaPar, int iter, float epsil,
                   float lipschitz_const, int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ);

/* replaces TV_SB_GPU_main, src/Core/regularisers_GPU/TV_SB_GPU_core.h:8 */
int TV_SB_GPU_main(float *Input, float *Output, float *infovector, float mu, int iter, float epsil, int methodTV,
                   int gpu_device, int dimX, int dimY, int dimZ);

/* replaces TGV_GPU_main, src/Core/regularisers_GPU/TGV_GPU_core.h:8.
 * dimX is the fastest axis, as for every other entry point (the reference's
 * Python passes TGV's dims reversed, src/Python/ccpi/filters/TV.py:722-725). */
int TGV_GPU_main(float *U0, float *U, float *infovector, float lambda, float alpha1, float alpha0,
                 int iterationsNumb, float L2, float epsil, int gpu_device, int dimX, int dimY, int dimZ);

/* replaces NonlDiff_GPU_main, src/Core/regularisers_GPU/NonlDiff_GPU_core.h:6.
 * Deterministic Jacobi sweeps (the reference updates in place, racing).
 * penaltytype outside 1..5 with sigmaPar != 0 returns -2. */
int NonlDiff_GPU_main(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                      int iterationsNumb, float tau, int penaltytype, float epsil, int gpu_device, int N, int M,
                      int Z);

/* replaces Diffus4th_GPU_main, src/Core/regularisers_GPU/Diffus_4thO_GPU_core.h:6 */
int Diffus4th_GPU_main(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                       int iterationsNumb, float tau, float epsil, int gpu_device, int N, int M, int Z);

/* replaces LLT_ROF_GPU_main, src/Core/regularisers_GPU/LLT_ROF_GPU_core.h:6 */
int LLT_ROF_GPU_main(float *Input, float *Output, float *infovector, float lambdaROF, float lambdaLLT,
                     int iterationsNumb, float tau, float epsil, int gpu_device, int N, int M, int Z);

/* replaces dTV_FGP_GPU_main, src/Core/regularisers_GPU/dTV_FGP_GPU_core.h:7.
 * U_prev of iteration 0 is zero, as in TV_FGP_GPU_main. */
int dTV_FGP_GPU_main(float *Input, float *InputRef, float *Output, float *infovector, float lambdaPar, int iter,
                     float epsil, float eta, int methodTV, int nonneg, int gpu_device, int dimX, int dimY, int dimZ);

/* ---------------------------------------------------------------------------
 * Reference C-OMP ABI.  Same argument lists and return type as the
 * reference; the work runs on GPU CILREG_GPU_DEVICE (environment, default 0).
 * Returns 0.0f or a negative status.
 * ------------------------------------------------------------------------- */

/* replaces TV_ROF_CPU_main, src/Core/regularisers_CPU/ROF_TV_core.h:48 (lambda_is_arr supported) */
float TV_ROF_CPU_main(float *Input, float *Output, float *infovector, float *lambdaPar, int lambda_is_arr,
                      int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ);

/* replaces TV_FGP_CPU_main, src/Core/regularisers_CPU/FGP_TV_core.h:51 */
float TV_FGP_CPU_main(float *Input, float *Output, float *infovector, float lambdaPar, int iterationsNumb,
                      float epsil, int methodTV, int nonneg, int dimX, int dimY, int dimZ);

/* replaces PDTV_CPU_main, src/Core/regularisers_CPU/PD_TV_core.h:50 */
float PDTV_CPU_main(float *Input, float *U, float *infovector, float lambdaPar, int iterationsNumb, float epsil,
                    float lipschitz_const, int methodTV, int nonneg, int dimX, int dimY, int dimZ);

/* replaces SB_TV_CPU_main, src/Core/regularisers_CPU/SB_TV_core.h:48 */
float SB_TV_CPU_main(float *Input, float *Output, float *infovector, float mu, int iter, float epsil, int methodTV,
                     int dimX, int dimY, int dimZ);

/* replaces TGV_main, src/Core/regularisers_CPU/TGV_core.h:53 */
float TGV_main(float *U0, float *U, float *infovector, float lambda, float alpha1, float alpha0, int iter, float L2,
               float epsil, int dimX, int dimY, int dimZ);

/* replaces Diffusion_CPU_main, src/Core/regularisers_CPU/Diffusion_core.h:54 (Jacobi order) */
float Diffusion_CPU_main(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                         int iterationsNumb, float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ);

/* replaces Diffus4th_CPU_main, src/Core/regularisers_CPU/Diffus4th_order_core.h:50 */
float Diffus4th_CPU_main(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                         int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ);

/* replaces LLT_ROF_CPU_main, src/Core/regularisers_CPU/LLT_ROF_core.h:52 */
float LLT_ROF_CPU_main(float *Input, float *Output, float *infovector, float lambdaROF, float lambdaLLT,
                       int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ);

/* replaces dTV_FGP_CPU_main, src/Core/regularisers_CPU/FGP_dTV_core.h:56 */
float dTV_FGP_CPU_main(float *Input, float *InputRef, float *Output, float *infovector, float lambdaPar,
                       int iterationsNumb, float epsil, float eta, int methodTV, int nonneg, int dimX, int dimY,
                       int dimZ);

/* replace TV_energy2D / TV_energy3D, src/Core/regularisers_CPU/utils.h:30-31.
 * Writes E_val[0] and returns it; type 1: 2 lambda TV(U) + |U - U0|^2, type 2:
 * 2 lambda TV(U).  Terms summed in double (the reference sums sequentially in
 * float).  On failure E_val[0] and the return value are NaN and
 * cilreg_last_error() says why. */
float TV_energy2D(float *U, float *U0, float *E_val, float lambda, int type, int dimX, int dimY);
float TV_energy3D(float *U, float *U0, float *E_val, float lambda, int type, int dimX, int dimY, int dimZ);

/* ---------------------------------------------------------------------------
 * Device-pointer API.  d_in / d_out are distinct device buffers of
 * dimX*dimY*dimZ floats on the current device; `stream` is a cudaStream_t
 * (NULL = legacy default stream).  Scratch comes from the device's
 * stream-ordered memory pool.  The call returns after the result is in d_out.
 * These mirror the device-array API of the reference's
 * src/Python/ccpi/filters/regularisersCuPy.py:35-40,130-138, extended to all
 * seven regularisers; argument meanings follow the *_CPU_main lists above.
 * ------------------------------------------------------------------------- */

/* d_lambda: optional per-voxel lambda (device), overriding lambdaPar (ROF_TV_core.c:280) */
int cilreg_rof_tv_dev(const float *d_in, float *d_out, float *infovector, const float *d_lambda, float lambdaPar,
                      int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void *stream);
int cilreg_fgp_tv_dev(const float *d_in, float *d_out, float *infovector, float lambdaPar, int iters, float epsil,
                      int methodTV, int nonneg, int dimX, int dimY, int dimZ, void *stream);
int cilreg_pd_tv_dev(const float *d_in, float *d_out, float *infovector, float lambdaPar, int iters, float epsil,
                     float lipschitz_const, int methodTV, int nonneg, int dimX, int dimY, int dimZ, void *stream);
int cilreg_sb_tv_dev(const float *d_in, float *d_out, float *infovector, float mu, int iters, float epsil,
                     int methodTV, int dimX, int dimY, int dimZ, void *stream);
int cilreg_tgv_dev(const float *d_in, float *d_out, float *infovector, float lambdaPar, float alpha1, float alpha0,
                   int iters, float L2, float epsil, int dimX, int dimY, int dimZ, void *stream);
int cilreg_ndf_dev(const float *d_in, float *d_out, float *infovector, float lambdaPar, float sigmaPar, int iters,
                   float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ, void *stream);
int cilreg_diff4th_dev(const float *d_in, float *d_out, float *infovector, float lambdaPar, float sigmaPar,
                       int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void *stream);
int cilreg_llt_rof_dev(const float *d_in, float *d_out, float *infovector, float lambdaROF, float lambdaLLT,
                       int iters, float tau, float epsil, int dimX, int dimY, int dimZ, void *stream);
/* d_ref: the reference image (device) of FGP-dTV */
int cilreg_dtv_fgp_dev(const float *d_in, const float *d_ref, float *d_out, float *infovector, float lambdaPar,
                       int iters, float epsil, float eta, int methodTV, int nonneg, int dimX, int dimY, int dimZ,
                       void *stream);
/* TV energy of device arrays; E_val is a host pointer to one float */
int cilreg_tv_energy_dev(const float *d_u, const float *d_u0, float *E_val, float lambda, int type, int dimX,
                         int dimY, int dimZ, void *stream);

/* ---------------------------------------------------------------------------
 * Batched API (no counterpart in the reference, whose callers loop over
 * volumes, e.g. demos/multi_gpu.py).  nvol volumes of any shapes (all 2D or
 * all 3D): d_in/d_out are host arrays of nvol device pointers, dims holds
 * (dimX, dimY, dimZ) per volume, lambdas one value per volume, infovectors
 * (host, may be NULL) 2 floats per volume.  Every volume follows its own
 * stopping rule.  All volumes advance together: one kernel launch per
 * iteration over all volumes' tiles, and by default the whole iteration loop
 * is one CUDA graph launch (CILREG_BATCH_GRAPH=0 disables the graph;
 * CILREG_BATCH_AUTOTUNE=1 times candidate z chunks of the FGP kernel on the
 * batch and keeps the choice, also in the file CILREG_AUTOTUNE_CACHE).  The
 * call returns when every output is written.  Results equal those of the
 * single-volume calls (FGP bit for bit, TGV to the last bits).
 * ------------------------------------------------------------------------- */
int cilreg_fgp_tv_batch_dev(int nvol, const float *const *d_in, float *const *d_out, const int *dims,
                            const float *lambdas, int iters, float epsil, int methodTV, int nonneg, float *infovectors,
                            void *stream);
int cilreg_tgv_batch_dev(int nvol, const float *const *d_in, float *const *d_out, const int *dims,
                         const float *lambdas, float alpha1, float alpha0, int iters, float L2, float epsil,
                         float *infovectors, void *stream);

/* ---------------------------------------------------------------------------
 * Differentiation (no counterpart in the reference).  Vector-Jacobian product
 * of the unrolled FGP-TV map y = FGP(f, lambda) with `iters` iterations and no
 * stopping rule (the map cilreg_fgp_tv_dev computes with epsil = 0): given
 * d_ybar = dL/dy it writes d_inbar = dL/df (device) and *lambar = dL/dlambda
 * (host).  Forward states are stored every `checkpoint` iterations (1..64) and
 * each segment is recomputed before its reverse sweep.
 * ------------------------------------------------------------------------- */
int cilreg_fgp_tv_vjp_dev(const float *d_in, const float *d_ybar, float *d_inbar, double *lambar, float lambdaPar,
                          int iters, int methodTV, int nonneg, int checkpoint, int dimX, int dimY, int dimZ,
                          void *stream);
/* The same for the unrolled ROF-TV map y = ROF(f, lambda) with scalar lambda,
 * time step tau and `iters` iterations (the map cilreg_rof_tv_dev computes with
 * d_lambda = NULL and epsil = 0); `checkpoint` >= 1 iterations per segment
 * (one stored volume per segment plus checkpoint - 1 for the recomputed
 * segment). */
int cilreg_rof_tv_vjp_dev(const float *d_in, const float *d_ybar, float *d_inbar, double *lambar, float lambdaPar,
                          int iters, float tau, int checkpoint, int dimX, int dimY, int dimZ, void *stream);

/* ---------------------------------------------------------------------------
 * Prox sessions (no counterpart in the reference, which discards all state at
 * the end of every call).  A session holds a regulariser's state on the
 * device across the outer iterations of a proximal-splitting solver:
 *   alg 0 ROF-TV  params {lambda, tau}            keeps the previous prox output
 *   alg 1 FGP-TV  params {lambda, methodTV, nonneg} keeps the dual iterates P
 *   alg 2 SB-TV   params {mu, methodTV}           keeps the split/Bregman D, B
 *   alg 3 NDF     params {lambda, sigma, tau, penalty} keeps the previous output
 * cilreg_prox_session_bytes gives the device memory one session needs (state
 * plus the transient scratch of a prox call), for admission control.
 * _prox runs `iters` warm-started iterations of the regulariser on d_in;
 * _fista solves min_x 1/2 ||x - f||^2 + R(x) with `outer` FISTA steps of
 * gradient step `step`, each prox being `inner` warm-started iterations, and
 * writes x to d_x.  A session is used by one host thread at a time.
 * ------------------------------------------------------------------------- */
typedef struct cilreg_session cilreg_session;
long long cilreg_prox_session_bytes(int alg, int dimX, int dimY, int dimZ);
int cilreg_prox_session_create(cilreg_session **session, int alg, const float *params, int nparams, int dimX,
                               int dimY, int dimZ, void *stream);
int cilreg_prox_session_prox(cilreg_session *session, const float *d_in, float *d_out, int iters, float epsil,
                             float *infovector, void *stream);
int cilreg_prox_session_fista(cilreg_session *session, const float *d_f, float *d_x, int outer, int inner, float step,
                              void *stream);
/* ADMM (scaled form) on min_x 1/2 ||w^(1/2) (x - f)||^2 + rho R(x), the
 * session's regulariser being the prox of R (so that its parameters already
 * carry the 1/rho): z = f, u = 0; per outer step x = (w f + rho (z - u)) /
 * (w + rho), z = prox(x + u) (`inner` warm-started iterations), u += x - z;
 * writes z to d_x.  d_w holds per-voxel data weights (a mask for inpainting)
 * or is NULL for w = 1.  The splitting of the reference's reconstruction demo
 * (demos/SoftwareX_supp/Demo_SimulData_Recon_SX.py:155-172) with the forward
 * operator a diagonal. */
int cilreg_prox_session_admm(cilreg_session *session, const float *d_f, const float *d_w, float *d_x, int outer,
                             int inner, float rho, void *stream);
/* PDHG (Chambolle-Pock with K = I) on min_x 1/2 ||w^(1/2) (x - f)||^2 +
 * sigma R(x), the session's regulariser being the prox of R: x = xbar = f,
 * y = 0; per outer step q = y / sigma + xbar, y = sigma (q - prox(q)),
 * x+ = (x - tau y + tau w f) / (1 + tau w), xbar = 2 x+ - x; writes x to d_x.
 * Convergent for tau sigma <= 1. */
int cilreg_prox_session_pdhg(cilreg_session *session, const float *d_f, const float *d_w, float *d_x, int outer,
                             int inner, float tau, float sigma, void *stream);
/* Register a host flag (or NULL to remove it) that the outer loops above read
 * before each outer step; while one is registered every outer step is waited
 * for, and a nonzero flag ends the loop with -5 (cancelled). */
int cilreg_prox_session_set_cancel(cilreg_session *session, const volatile int *flag);
int cilreg_prox_session_destroy(cilreg_session *session, void *stream);

/* Host-side fault injection for tests (no counterpart in the reference): the
 * next n device allocations the library makes (scratch and prox sessions)
 * fail with -4 as if the device were full; 0 clears it. */
int cilreg_debug_fail_allocations(int n);

/* No counterpart in the reference.  ROF-TV like cilreg_rof_tv_dev, but the
 * call allocates no device memory at all, for callers that cannot allocate
 * when they regularise: a framework that has already claimed the GPU's memory
 * for its own caching allocator or budget, or a real-time pipeline that
 * forbids allocation after start-up.  Its scratch is one fixed device array
 * of 68 MiB inside the library, held by every GPU that loads it until exit.
 * Limits: at most 2^24 voxels (e.g. 256^3 or 4096^2), otherwise -2; with
 * epsil != 0 at most 2^18 reduction blocks.  All calls share the array:
 * calls whose GPU work overlaps race and must be serialised by the caller.
 * The first call on a device looks up the array's address on that device.
 * A call waits for its stream before it returns, so it cannot be captured
 * into a CUDA graph; with epsil != 0 it reads the stop flag every twentieth
 * iteration and stops enqueueing once the rule has fired. */
int cilreg_rof_tv_dev_noalloc(const float *d_in, float *d_out, float *infovector, const float *d_lambda,
                              float lambdaPar, int iters, float tau, float epsil, int dimX, int dimY, int dimZ,
                              void *stream);

/* ---------------------------------------------------------------------------
 * Library information (no counterpart in the reference).
 * ------------------------------------------------------------------------- */
const char *cilreg_last_error(void);
const char *cilreg_version(void);
int cilreg_device_count(void);
/* number of kernels this library has launched in the process so far */
long long cilreg_launch_count(void);
/* Scratch memory is taken from the device's stream-ordered pool and kept
 * there when a call returns, so that later calls do not map it again; a call
 * that finds the device full first hands the pool's unused memory back and
 * retries.  This waits for all work on the device, then hands back what the
 * pool holds unused (for callers that share the device with another
 * allocator).  0 or a negative status. */
int cilreg_release_cached(int gpu_device);
/* Self-test of the bounded waits of the kernels that stage their inputs by
 * tensor copies: one CTA waits on an mbarrier whose 16 expected bytes never
 * arrive (no copy is issued).  *ran_out = 1 when the wait gave up after its
 * try limit, as it must, and the device then still ran a kernel.  0 or a
 * negative status. */
int cilreg_selftest_wait_limit(int gpu_device, int *ran_out);
/* Self-test of the bounded dependency waits of the persistent batched FGP
 * kernel: a launch whose work items all wait for an iteration that is never
 * released.  *ran_out = 1 when the waits gave up after their poll limit and
 * the call reported it, and the device then still ran work.  0 or a
 * negative status. */
int cilreg_selftest_batch_wait(int gpu_device, int *ran_out);
/* Self-test of the kernels' reciprocal (the approximate reciprocal with one
 * Newton-Raphson step, used by the two-voxel fourth-order diffusion kernel):
 * approx[i] = that reciprocal of the host array x[i], ieee[i] = CUDA's
 * correctly rounded reciprocal of x[i], for 1 <= n <= 2^30.  0 or a negative
 * status. */
int cilreg_selftest_reciprocal(int gpu_device, const float *x, float *approx, float *ieee, long long n);

#ifdef __cplusplus
}
#endif

#endif /* CILREG_GB300_H */
