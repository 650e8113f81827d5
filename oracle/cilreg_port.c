/*
 * ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, CPU restatement of the seven iterative proximal regularisers of
 * the CCPi Regularisation Toolkit (C-OMP path, FP32), of LLT-ROF and FGP-dTV
 * and of the TV energy diagnostic.  It exists so that the
 * GPU product can be checked against the reference's arithmetic on the GPU
 * machine, where the reference sources are not available.  Only the test
 * suite, the smoke check and the CPU-baseline leg of the benchmark load it;
 * the product library never links or calls it.
 *
 * Every routine follows the reference's loop order and floating-point
 * evaluation order (including the places where the reference promotes to
 * double) so that, built with -ffp-contract=off, it reproduces the
 * reference bit for bit on x86-64.  Citations are to files of the reference
 * project (src/Core/regularisers_CPU/...).
 *
 * Deliberate, documented difference: on an axis of length 1 the reference's
 * mirrored neighbour index (i+1 -> i-1) points outside the array; here the
 * mirrored neighbour of a length-1 axis is the voxel itself.  No other
 * behaviour differs.
 *
 * Non-linear diffusion is provided in two update orders:
 *   jacobi=1  every voxel reads the previous sweep only (the GPU semantics);
 *   jacobi=0  lexicographic in-place sweep, identical to the reference run
 *             with one OpenMP thread (Diffusion_core.c:282-413).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef long idx_t;

/* ------------------------------------------------------------------ */
/* shared helpers                                                      */
/* ------------------------------------------------------------------ */

/* mirrored neighbours: hi(i)=i+1 (i-1 at the last index), lo(i)=i-1 (i+1 at 0) */
static inline idx_t nb_hi(idx_t i, idx_t n) { if (n == 1) return 0; return (i + 1 >= n) ? i - 1 : i + 1; }
static inline idx_t nb_lo(idx_t i, idx_t n) { if (n == 1) return 0; return (i - 1 < 0) ? i + 1 : i - 1; }

static inline int sgn_f(float x) { return (x > 0) - (x < 0); }

static void copy_arr(const float *a, float *b, idx_t n)
{
    idx_t j;
#pragma omp parallel for
    for (j = 0; j < n; j++) b[j] = a[j];
}

static float *zalloc(idx_t n) { return (float *)calloc((size_t)n, sizeof(float)); }

/* relative change used by every stopping rule: sequential FP32 sums
 * (e.g. FGP_TV_core.c:142-153) */
static float rel_change(const float *u, const float *uprev, idx_t n)
{
    float a = 0.0f, b = 0.0f;
    idx_t j;
    for (j = 0; j < n; j++) {
        a += powf(u[j] - uprev[j], 2);
        b += powf(u[j], 2);
    }
    return sqrtf(a) / sqrtf(b);
}

/* optional trace of every relative change the stopping rule evaluates, so a
 * test can tell a genuine stopping-iteration mismatch from a borderline one */
static float *g_trace = NULL;
static int g_trace_cap = 0, g_trace_len = 0;

void port_set_trace(float *buf, int cap)
{
    g_trace = buf;
    g_trace_cap = cap;
    g_trace_len = 0;
}

int port_trace_len(void) { return g_trace_len; }

/* stopping bookkeeping shared by all drivers: returns 1 when the loop must stop */
typedef struct { float re; int count; } stop_state;
static int stop_check(stop_state *s, const float *u, const float *uprev, idx_t n, float epsil)
{
    s->re = rel_change(u, uprev, n);
    if (g_trace && g_trace_len < g_trace_cap) g_trace[g_trace_len++] = s->re;
    if (s->re < epsil) s->count++;
    return s->count > 3;
}

/* ------------------------------------------------------------------ */
/* ROF-TV explicit gradient flow  (ROF_TV_core.c:50-317)               */
/* ------------------------------------------------------------------ */

/* 0.5*(sign(a)+sign(b))*min(|a|,|b|) — the minmod term of ROF_TV_core.c:132 */
static inline float rof_minmod(float a, float b)
{
    return (float)(0.5f * (sgn_f(a) + sgn_f(b)) * fmin(fabs(a), fabs(b)));
}

/* eps: 1e-8 for ROF-TV (ROF_TV_core.c:22), 1e-12 inside LLT-ROF (LLT_ROF_core.c:22) */
static void rof_fluxes(const float *A, float *D1, float *D2, float *D3, idx_t nx, idx_t ny, idx_t nz,
                       double eps)
{
    idx_t i, j, k;
    if (nz > 1) {
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t s = nx * ny, v = s * k + nx * j + i;
                    idx_t ip = nb_hi(i, nx), im = nb_lo(i, nx);
                    idx_t jp = nb_hi(j, ny), jm = nb_lo(j, ny);
                    idx_t kp = nb_hi(k, nz), km = nb_lo(k, nz);
                    float a = A[v];
                    float dyp = A[s * k + nx * jp + i] - a, dym = a - A[s * k + nx * jm + i];
                    float dxp = A[s * k + nx * j + ip] - a, dxm = a - A[s * k + nx * j + im];
                    float dzp = A[s * kp + nx * j + i] - a, dzm = a - A[s * km + nx * j + i];
                    float m, t1, t2, t3;
                    /* D1 (j axis): double sqrt as in ROF_TV_core.c:136 */
                    {
                        float d1 = dyp * dyp, d2, d3;
                        m = rof_minmod(dxp, dxm); d2 = m * m;
                        m = rof_minmod(dzp, dzm); d3 = m * m;
                        t1 = (float)sqrt(d1 + d2 + d3 + eps);
                        D1[v] = dyp / t1;
                    }
                    /* D2 (i axis): ROF_TV_core.c:194-200 */
                    {
                        float d1 = dxp * dxp, d2, d3;
                        m = rof_minmod(dyp, dym); d2 = m * m;
                        m = rof_minmod(dzp, dzm); d3 = m * m;
                        t2 = sqrtf((float)(d1 + d2 + d3 + eps));
                        D2[v] = dxp / t2;
                    }
                    /* D3 (k axis): ROF_TV_core.c:257-263 */
                    {
                        float d1 = dzp * dzp, d2, d3;
                        m = rof_minmod(dyp, dym); d2 = m * m;
                        m = rof_minmod(dxp, dxm); d3 = m * m;
                        t3 = sqrtf((float)(d1 + d2 + d3 + eps));
                        D3[v] = dzp / t3;
                    }
                }
    } else {
#pragma omp parallel for private(i)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = nx * j + i;
                idx_t ip = nb_hi(i, nx), im = nb_lo(i, nx);
                idx_t jp = nb_hi(j, ny), jm = nb_lo(j, ny);
                float a = A[v];
                float dyp = A[nx * jp + i] - a, dym = a - A[nx * jm + i];
                float dxp = A[nx * j + ip] - a, dxm = a - A[nx * j + im];
                float m, d1, d2;
                d1 = dyp * dyp; m = rof_minmod(dxp, dxm); d2 = m * m;
                D1[v] = dyp / sqrtf((float)(d1 + d2 + eps));
                d1 = dxp * dxp; m = rof_minmod(dyp, dym); d2 = m * m;
                D2[v] = dxp / sqrtf((float)(d1 + d2 + eps));
            }
    }
}

static void rof_update(const float *D1, const float *D2, const float *D3, float *U, const float *F,
                       const float *lam, int lam_is_arr, float tau, idx_t nx, idx_t ny, idx_t nz)
{
    idx_t i, j, k;
    if (nz > 1) {
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t s = nx * ny, v = s * k + nx * j + i;
                    float l = lam[v * lam_is_arr];
                    float dv1 = D1[v] - D1[s * k + nx * nb_lo(j, ny) + i];
                    float dv2 = D2[v] - D2[s * k + nx * j + nb_lo(i, nx)];
                    float dv3 = D3[v] - D3[s * nb_lo(k, nz) + nx * j + i];
                    U[v] += tau * (l * (dv1 + dv2 + dv3) - (U[v] - F[v]));
                }
    } else {
#pragma omp parallel for private(i)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = nx * j + i;
                float l = lam[v * lam_is_arr];
                float dv1 = D1[v] - D1[nx * nb_lo(j, ny) + i];
                float dv2 = D2[v] - D2[nx * j + nb_lo(i, nx)];
                U[v] += tau * (l * (dv1 + dv2) - (U[v] - F[v]));
            }
    }
}

/* u_init (optional) replaces Input as the starting iterate: the warm start of
 * a prox session, whose ROF and NDF proxes continue from the previous output */
static float rof_main(float *Input, float *Output, float *infovector, float *lambdaPar, int lambda_is_arr,
                      int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ, const float *u_init)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    idx_t nx = dimX, ny = dimY, nz = dimZ, n = nx * ny * nz;
    float *D1 = zalloc(n), *D2 = zalloc(n), *D3 = zalloc(n), *Uprev = NULL;
    stop_state st = {0.0f, 0};
    int it;
    copy_arr(u_init ? u_init : Input, Output, n);
    if (epsil != 0.0f) Uprev = zalloc(n);
    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        if (check) copy_arr(Output, Uprev, n);
        rof_fluxes(Output, D1, D2, D3, nx, ny, nz, 1.0e-8);
        rof_update(D1, D2, D3, Output, Input, lambdaPar, lambda_is_arr, tau, nx, ny, nz);
        if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    free(D1); free(D2); free(D3); free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

float port_TV_ROF(float *Input, float *Output, float *infovector, float *lambdaPar, int lambda_is_arr,
                  int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ)
{
    return rof_main(Input, Output, infovector, lambdaPar, lambda_is_arr, iterationsNumb, tau, epsil, dimX, dimY,
                    dimZ, NULL);
}

float port_TV_ROF_init(float *Input, float *Output, float *infovector, float lambdaPar, int iterationsNumb,
                       float tau, float epsil, int dimX, int dimY, int dimZ, const float *u_init)
{
    return rof_main(Input, Output, infovector, &lambdaPar, 0, iterationsNumb, tau, epsil, dimX, dimY, dimZ,
                    u_init);
}

/* ------------------------------------------------------------------ */
/* dual projections shared by FGP and PD  (utils.c:149-213)            */
/* ------------------------------------------------------------------ */
static void project_dual(float *P1, float *P2, float *P3, int methodTV, idx_t n)
{
    idx_t i;
    if (methodTV == 0) {
#pragma omp parallel for
        for (i = 0; i < n; i++) {
            float d = P3 ? powf(P1[i], 2) + powf(P2[i], 2) + powf(P3[i], 2) : powf(P1[i], 2) + powf(P2[i], 2);
            if (d > 1.0f) {
                float s = 1.0f / sqrtf(d);
                P1[i] = P1[i] * s;
                P2[i] = P2[i] * s;
                if (P3) P3[i] = P3[i] * s;
            }
        }
    } else {
#pragma omp parallel for
        for (i = 0; i < n; i++) {
            float a1 = (float)fabs(P1[i]), a2 = (float)fabs(P2[i]);
            if (a1 < 1.0f) a1 = 1.0f;
            if (a2 < 1.0f) a2 = 1.0f;
            P1[i] = P1[i] / a1;
            P2[i] = P2[i] / a2;
            if (P3) {
                float a3 = (float)fabs(P3[i]);
                if (a3 < 1.0f) a3 = 1.0f;
                P3[i] = P3[i] / a3;
            }
        }
    }
}

static void clamp_nonneg(float *U, idx_t n)
{
    idx_t j;
    for (j = 0; j < n; j++) if (U[j] < 0.0f) U[j] = 0.0f;
}

/* ------------------------------------------------------------------ */
/* FGP-TV  (FGP_TV_core.c:40-269)                                      */
/* ------------------------------------------------------------------ */
/* pstate (optional, na arrays of n floats back to back): the dual iterate a
 * previous call ended with.  R and P_prev start from it instead of zero (the
 * momentum restarts at t = 1, so the first R is exactly that P), and the last
 * P is written back to it: the warm start of a prox session. */
static float fgp_main(float *Input, float *Output, float *infovector, float lambdaPar, int iterationsNumb,
                      float epsil, int methodTV, int nonneg, int dimX, int dimY, int dimZ, float *pstate)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ > 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz, s = nx * ny;
    float *P[3] = {0}, *Pold[3] = {0}, *R[3] = {0}, *Uprev = NULL;
    int c, na = three ? 3 : 2, it;
    float tk = 1.0f, tkp1 = 1.0f;
    float multip = three ? (1.0f / (12.0f * lambdaPar)) : (1.0f / (8.0f * lambdaPar));
    stop_state st = {0.0f, 0};
    for (c = 0; c < na; c++) { P[c] = zalloc(n); Pold[c] = zalloc(n); R[c] = zalloc(n); }
    if (pstate)
        for (c = 0; c < na; c++) { copy_arr(pstate + c * n, R[c], n); copy_arr(pstate + c * n, Pold[c], n); }
    if (epsil != 0.0f) Uprev = zalloc(n);

    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        idx_t i, j, k;
        if (check) copy_arr(Output, Uprev, n);
        /* objective: U = f - lambda*div(R), zero flux below index 0 */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float b1 = (i == 0) ? 0.0f : R[0][v - 1];
                    float b2 = (j == 0) ? 0.0f : R[1][v - nx];
                    if (three) {
                        float b3 = (k == 0) ? 0.0f : R[2][v - s];
                        Output[v] = Input[v] - lambdaPar * (R[0][v] + R[1][v] + R[2][v] - b1 - b2 - b3);
                    } else {
                        Output[v] = Input[v] - lambdaPar * (R[0][v] + R[1][v] - b1 - b2);
                    }
                }
        if (nonneg == 1) clamp_nonneg(Output, n);
        /* gradient step: P = R + multip*(U - U[+1]), zero at the last index */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float g1 = (i == nx - 1) ? 0.0f : Output[v] - Output[v + 1];
                    float g2 = (j == ny - 1) ? 0.0f : Output[v] - Output[v + nx];
                    P[0][v] = R[0][v] + multip * g1;
                    P[1][v] = R[1][v] + multip * g2;
                    if (three) {
                        float g3 = (k == nz - 1) ? 0.0f : Output[v] - Output[v + s];
                        P[2][v] = R[2][v] + multip * g3;
                    }
                }
        project_dual(P[0], P[1], three ? P[2] : NULL, methodTV, n);
        tkp1 = (1.0f + sqrtf(1.0f + 4.0f * tk * tk)) * 0.5f;
        {
            float m = (tk - 1.0f) / tkp1;
#pragma omp parallel for
            for (i = 0; i < n; i++)
                for (c = 0; c < na; c++) R[c][i] = P[c][i] + m * (P[c][i] - Pold[c][i]);
        }
        if (three) {
            /* 3D: the stopping check precedes the P_prev copy (FGP_TV_core.c:142-158) */
            if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
            for (c = 0; c < na; c++) copy_arr(P[c], Pold[c], n);
            tk = tkp1;
        } else {
            for (c = 0; c < na; c++) copy_arr(P[c], Pold[c], n);
            tk = tkp1;
            if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
        }
    }
    if (pstate)
        for (c = 0; c < na; c++) copy_arr(P[c], pstate + c * n, n);
    for (c = 0; c < na; c++) { free(P[c]); free(Pold[c]); free(R[c]); }
    free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

float port_TV_FGP(float *Input, float *Output, float *infovector, float lambdaPar, int iterationsNumb,
                  float epsil, int methodTV, int nonneg, int dimX, int dimY, int dimZ)
{
    return fgp_main(Input, Output, infovector, lambdaPar, iterationsNumb, epsil, methodTV, nonneg, dimX, dimY, dimZ,
                    NULL);
}

float port_TV_FGP_warm(float *Input, float *Output, float *infovector, float lambdaPar, int iterationsNumb,
                       float epsil, int methodTV, int nonneg, int dimX, int dimY, int dimZ, float *pstate)
{
    return fgp_main(Input, Output, infovector, lambdaPar, iterationsNumb, epsil, methodTV, nonneg, dimX, dimY, dimZ,
                    pstate);
}

/* ------------------------------------------------------------------ */
/* PD-TV, Chambolle-Pock  (PD_TV_core.c:40-252)                        */
/* ------------------------------------------------------------------ */
float port_PDTV(float *Input, float *U, float *infovector, float lambdaPar, int iterationsNumb, float epsil,
                float lipschitz_const, int methodTV, int nonneg, int dimX, int dimY, int dimZ)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ > 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz, s = nx * ny;
    float tau = lambdaPar * 0.1f;
    float sigma = (float)(1.0 / (lipschitz_const * tau));
    float theta = 1.0f;
    float lt = tau / lambdaPar;
    float *Uold = zalloc(n), *P1 = zalloc(n), *P2 = zalloc(n), *P3 = three ? zalloc(n) : NULL;
    stop_state st = {0.0f, 0};
    int it;
    copy_arr(Input, U, n);
    for (it = 0; it < iterationsNumb; it++) {
        idx_t i, j, k;
        /* dual ascent with mirrored forward differences */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    P1[v] += sigma * (U[s * k + nx * j + nb_hi(i, nx)] - U[v]);
                    P2[v] += sigma * (U[s * k + nx * nb_hi(j, ny) + i] - U[v]);
                    if (three) P3[v] += sigma * (U[s * nb_hi(k, nz) + nx * j + i] - U[v]);
                }
        if (nonneg == 1) clamp_nonneg(U, n);
        project_dual(P1, P2, P3, methodTV, n);
        copy_arr(U, Uold, n);
        /* primal step with backward divergence, P[-1] = 0 */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float q1 = (i == 0) ? -P1[v] : -(P1[v] - P1[v - 1]);
                    float q2 = (j == 0) ? -P2[v] : -(P2[v] - P2[v - nx]);
                    float dv;
                    if (three) {
                        float q3 = (k == 0) ? -P3[v] : -(P3[v] - P3[v - s]);
                        dv = q1 + q2 + q3;
                    } else {
                        dv = q1 + q2;
                    }
                    U[v] = (float)((U[v] - tau * dv + lt * Input[v]) / (1.0 + lt));
                }
        if ((epsil != 0.0f) && (it % 5 == 0) && stop_check(&st, U, Uold, n, epsil)) break;
#pragma omp parallel for
        for (i = 0; i < n; i++) U[i] += theta * (U[i] - Uold[i]);
    }
    free(Uold); free(P1); free(P2); free(P3);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Split-Bregman TV  (SB_TV_core.c:38-371)                             */
/* ------------------------------------------------------------------ */
static void sb_jacobi(float *U, const float *A, const float *Up, float *const *D, float *const *B,
                      int three, idx_t nx, idx_t ny, idx_t nz, float lambda, float mu)
{
    idx_t i, j, k, s = nx * ny;
    float norm = three ? 1.0f / (mu + 6.0f * lambda) : 1.0f / (mu + 4.0f * lambda);
#pragma omp parallel for private(i, j)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                idx_t xi = s * k + nx * j + nb_lo(i, nx), xo = s * k + nx * j + nb_hi(i, nx);
                idx_t yi = s * k + nx * nb_lo(j, ny) + i, yo = s * k + nx * nb_hi(j, ny) + i;
                float sum;
                if (three) {
                    idx_t zi = s * nb_lo(k, nz) + nx * j + i, zo = s * nb_hi(k, nz) + nx * j + i;
                    float dval = D[0][xi] - D[0][v] + D[1][yi] - D[1][v] + D[2][zi] - D[2][v];
                    float bval = -B[0][xi] + B[0][v] - B[1][yi] + B[1][v] - B[2][zi] + B[2][v];
                    sum = dval + bval;
                    sum += Up[xo] + Up[xi] + Up[yo] + Up[yi] + Up[zo] + Up[zi];
                } else {
                    sum = D[0][xi] - D[0][v] + D[1][yi] - D[1][v] - B[0][xi] + B[0][v] - B[1][yi] + B[1][v];
                    sum += Up[xo] + Up[xi] + Up[yo] + Up[yi];
                }
                sum *= lambda;
                sum += mu * A[v];
                U[v] = norm * sum;
            }
}

static void sb_shrink_bregman(const float *U, float *const *D, float *const *B, int three, int aniso,
                              idx_t nx, idx_t ny, idx_t nz, float lambda)
{
    idx_t i, j, k, s = nx * ny;
    float dl = 1.0f / lambda;
    int c, na = three ? 3 : 2;
    /* shrinkage (SB_TV_core.c:284-352) */
#pragma omp parallel for private(i, j, c)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                float g[3];
                g[0] = (U[s * k + nx * j + nb_hi(i, nx)] - U[v]) + B[0][v];
                g[1] = (U[s * k + nx * nb_hi(j, ny) + i] - U[v]) + B[1][v];
                g[2] = three ? (U[s * nb_hi(k, nz) + nx * j + i] - U[v]) + B[2][v] : 0.0f;
                if (aniso) {
                    for (c = 0; c < na; c++) {
                        float m = fabsf(g[c]) - dl;
                        if (m < 0.0f) m = 0.0f;
                        D[c][v] = (g[c] != 0.0f) ? (g[c] / fabsf(g[c])) * m : 0.0f;
                    }
                } else {
                    float den = three ? sqrtf(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) : sqrtf(g[0] * g[0] + g[1] * g[1]);
                    float m = den - dl;
                    if (m < 0) m = 0.0f;
                    for (c = 0; c < na; c++) D[c][v] = (den != 0.0f) ? m * (g[c] / den) : 0.0f;
                }
            }
    /* Bregman update (SB_TV_core.c:353-371) */
#pragma omp parallel for private(i, j)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                B[0][v] += (U[s * k + nx * j + nb_hi(i, nx)] - U[v]) - D[0][v];
                B[1][v] += (U[s * k + nx * nb_hi(j, ny) + i] - U[v]) - D[1][v];
                if (three) B[2][v] += (U[s * nb_hi(k, nz) + nx * j + i] - U[v]) - D[2][v];
            }
}

/* dbstate (optional, 2*na arrays of n floats: D components then B
 * components): the split and Bregman variables a previous call ended with;
 * they replace the zero start and receive the final D, B. */
static float sb_main(float *Input, float *Output, float *infovector, float mu, int iter, float epsil, int methodTV,
                     int dimX, int dimY, int dimZ, float *dbstate)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ != 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz;
    float lambda;
    float *Uprev = zalloc(n), *D[3] = {0}, *B[3] = {0};
    int c, na = three ? 3 : 2, it;
    stop_state st = {0.0f, 0};
    mu = 1.0f / mu;
    lambda = 2.0f * mu;
    for (c = 0; c < na; c++) { D[c] = zalloc(n); B[c] = zalloc(n); }
    if (dbstate)
        for (c = 0; c < na; c++) { copy_arr(dbstate + c * n, D[c], n); copy_arr(dbstate + (na + c) * n, B[c], n); }
    copy_arr(Input, Output, n);
    for (it = 0; it < iter; it++) {
        copy_arr(Output, Uprev, n);
        sb_jacobi(Output, Input, Uprev, D, B, three, nx, ny, nz, lambda, mu);
        copy_arr(Output, Uprev, n);
        sb_jacobi(Output, Input, Uprev, D, B, three, nx, ny, nz, lambda, mu);
        sb_shrink_bregman(Output, D, B, three, methodTV == 1, nx, ny, nz, lambda);
        if ((epsil != 0.0f) && (it % 5 == 0) && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    if (dbstate)
        for (c = 0; c < na; c++) { copy_arr(D[c], dbstate + c * n, n); copy_arr(B[c], dbstate + (na + c) * n, n); }
    for (c = 0; c < na; c++) { free(D[c]); free(B[c]); }
    free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

float port_SB_TV(float *Input, float *Output, float *infovector, float mu, int iter, float epsil, int methodTV,
                 int dimX, int dimY, int dimZ)
{
    return sb_main(Input, Output, infovector, mu, iter, epsil, methodTV, dimX, dimY, dimZ, NULL);
}

float port_SB_TV_warm(float *Input, float *Output, float *infovector, float mu, int iter, float epsil,
                      int methodTV, int dimX, int dimY, int dimZ, float *dbstate)
{
    return sb_main(Input, Output, infovector, mu, iter, epsil, methodTV, dimX, dimY, dimZ, dbstate);
}

/* ------------------------------------------------------------------ */
/* TGV (second order), primal-dual  (TGV_core.c:43-568)                */
/* ------------------------------------------------------------------ */

/* backward difference with the three-case boundary of TGV_core.c:286-292 */
static inline float tgv_bwd(const float *X, idx_t v, idx_t stride, idx_t i, idx_t n)
{
    if (i == 0) return X[v];
    if (i == n - 1) return -X[v - stride];
    return X[v] - X[v - stride];
}

float port_TGV(float *U0, float *U, float *infovector, float lambda, float alpha1, float alpha0, int iter,
               float L2, float epsil, int dimX, int dimY, int dimZ)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ != 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz, s = nx * ny;
    int np = three ? 3 : 2, nq = three ? 6 : 3, c, it;
    float tau = (float)pow(L2, -0.5), sigma = (float)pow(L2, -0.5);
    float *P[3] = {0}, *Q[6] = {0}, *V[3] = {0}, *Vold[3] = {0}, *Uold = zalloc(n);
    stop_state st = {0.0f, 0};
    copy_arr(U0, U, n);
    for (c = 0; c < np; c++) { P[c] = zalloc(n); V[c] = zalloc(n); Vold[c] = zalloc(n); }
    for (c = 0; c < nq; c++) Q[c] = zalloc(n);

    for (it = 0; it < iter; it++) {
        idx_t i, j, k;
        /* dual P: P += sigma*(grad U - V), only -V at the last index; then |P|<=alpha1 */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    if (i == nx - 1) P[0][v] += sigma * (-V[0][v]);
                    else P[0][v] += sigma * ((U[v + 1] - U[v]) - V[0][v]);
                    if (j == ny - 1) P[1][v] += sigma * (-V[1][v]);
                    else P[1][v] += sigma * ((U[v + nx] - U[v]) - V[1][v]);
                    if (three) {
                        if (k == nz - 1) P[2][v] += sigma * (-V[2][v]);
                        else P[2][v] += sigma * ((U[v + s] - U[v]) - V[2][v]);
                    }
                }
#pragma omp parallel for
        for (i = 0; i < n; i++) {
            float g = three ? sqrtf(P[0][i] * P[0][i] + P[1][i] * P[1][i] + P[2][i] * P[2][i]) / alpha1
                            : sqrtf(P[0][i] * P[0][i] + P[1][i] * P[1][i]) / alpha1;
            if (g > 1.0f) for (c = 0; c < np; c++) P[c][i] /= g;
        }
        /* dual Q: Q += sigma*sym_grad(V), zero at the last index; then Frobenius <= alpha0 */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    if (three) {
                        float q1 = 0, q11 = 0, q33 = 0, q2 = 0, q22 = 0, q55 = 0, q3 = 0, q44 = 0, q66 = 0;
                        if (i != nx - 1) { q1 = V[0][v + 1] - V[0][v]; q11 = V[1][v + 1] - V[1][v]; q33 = V[2][v + 1] - V[2][v]; }
                        if (j != ny - 1) { q2 = V[1][v + nx] - V[1][v]; q22 = V[0][v + nx] - V[0][v]; q55 = V[2][v + nx] - V[2][v]; }
                        if (k != nz - 1) { q3 = V[2][v + s] - V[2][v]; q44 = V[0][v + s] - V[0][v]; q66 = V[1][v + s] - V[1][v]; }
                        Q[0][v] += sigma * (q1);
                        Q[1][v] += sigma * (q2);
                        Q[2][v] += sigma * (q3);
                        Q[3][v] += sigma * (0.5f * (q11 + q22));
                        Q[4][v] += sigma * (0.5f * (q33 + q44));
                        Q[5][v] += sigma * (0.5f * (q55 + q66));
                    } else {
                        float q1 = 0, q11 = 0, q2 = 0, q22 = 0;
                        if (i != nx - 1) { q1 = V[0][v + 1] - V[0][v]; q11 = V[1][v + 1] - V[1][v]; }
                        if (j != ny - 1) { q2 = V[1][v + nx] - V[1][v]; q22 = V[0][v + nx] - V[0][v]; }
                        Q[0][v] += sigma * (q1);
                        Q[1][v] += sigma * (q2);
                        Q[2][v] += sigma * (0.5f * (q11 + q22));
                    }
                }
#pragma omp parallel for
        for (i = 0; i < n; i++) {
            float g;
            if (three)
                g = sqrtf(Q[0][i] * Q[0][i] + Q[1][i] * Q[1][i] + Q[2][i] * Q[2][i] + 2.0f * Q[3][i] * Q[3][i] +
                          2.0f * Q[4][i] * Q[4][i] + 2.0f * Q[5][i] * Q[5][i]);
            else
                g = sqrtf(Q[0][i] * Q[0][i] + Q[1][i] * Q[1][i] + 2 * Q[2][i] * Q[2][i]);
            g = g / alpha0;
            if (g > 1.0f) for (c = 0; c < nq; c++) Q[c][i] /= g;
        }
        copy_arr(U, Uold, n);
        /* primal U: proximal step on the divergence of P */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float dv = tgv_bwd(P[0], v, 1, i, nx) + tgv_bwd(P[1], v, nx, j, ny);
                    if (three) dv = dv + tgv_bwd(P[2], v, s, k, nz);
                    U[v] = (lambda * (U[v] + tau * dv) + tau * U0[v]) / (lambda + tau);
                }
#pragma omp parallel for
        for (i = 0; i < n; i++) U[i] = 2.0f * U[i] - Uold[i];
        for (c = 0; c < np; c++) copy_arr(V[c], Vold[c], n);
        /* primal V: V += tau*(P + div Q) */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    if (three) {
                        float q1 = tgv_bwd(Q[0], v, 1, i, nx), q4x = tgv_bwd(Q[3], v, 1, i, nx), q5x = tgv_bwd(Q[4], v, 1, i, nx);
                        float q2 = tgv_bwd(Q[1], v, nx, j, ny), q4y = tgv_bwd(Q[3], v, nx, j, ny), q6y = tgv_bwd(Q[5], v, nx, j, ny);
                        float q6z = tgv_bwd(Q[5], v, s, k, nz), q5z = tgv_bwd(Q[4], v, s, k, nz), q3 = tgv_bwd(Q[2], v, s, k, nz);
                        float d1 = q1 + q4y + q5z, d2 = q4x + q2 + q6z, d3 = q5x + q6y + q3;
                        V[0][v] += tau * (P[0][v] + d1);
                        V[1][v] += tau * (P[1][v] + d2);
                        V[2][v] += tau * (P[2][v] + d3);
                    } else {
                        float q1 = tgv_bwd(Q[0], v, 1, i, nx), q3x = tgv_bwd(Q[2], v, 1, i, nx);
                        float q2 = tgv_bwd(Q[1], v, nx, j, ny), q3y = tgv_bwd(Q[2], v, nx, j, ny);
                        float d1 = q1 + q3y, d2 = q3x + q2;
                        V[0][v] += tau * (P[0][v] + d1);
                        V[1][v] += tau * (P[1][v] + d2);
                    }
                }
#pragma omp parallel for private(c)
        for (i = 0; i < n; i++)
            for (c = 0; c < np; c++) V[c][i] = 2.0f * V[c][i] - Vold[c][i];
        if ((epsil != 0.0f) && (it % 5 == 0) && stop_check(&st, U, Uold, n, epsil)) break;
    }
    for (c = 0; c < np; c++) { free(P[c]); free(V[c]); free(Vold[c]); }
    for (c = 0; c < nq; c++) free(Q[c]);
    free(Uold);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

/* ------------------------------------------------------------------ */
/* (non)linear diffusion  (Diffusion_core.c:53-413)                    */
/* ------------------------------------------------------------------ */

/* edge-stopping function applied to one neighbour difference */
static inline float ndf_flux(float d, float sg, int penalty)
{
    switch (penalty) {
    case 1:
        return (fabs(d) > sg) ? (float)sgn_f(d) : d / sg;
    case 2:
        return d / (1.0f + powf((d / sg), 2));
    case 3:
        return (fabs(d) <= sg) ? d * powf((1.0f - powf((d / sg), 2)), 2) : 0.0f;
    case 4:
        return (fabs(d) > sg) ? 0.0f : d;
    case 5:
        if (fabs(d) <= 2.0f * sg) return (fabs(d) > sg) ? (float)sgn_f(d) : d / sg;
        return 0.0f;
    default:
        return d;
    }
}

/* one explicit sweep; reads Src, writes Dst (Src==Dst gives the in-place lexicographic order) */
static void ndf_sweep(const float *F, const float *Src, float *Dst, float lambda, float sg, float tau, int penalty,
                      int linear, idx_t nx, idx_t ny, idx_t nz, int serial)
{
    idx_t i, j, k, s = nx * ny;
    int three = nz > 1;
#pragma omp parallel for private(i, j) if (!serial)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                float c = Src[v];
                float e1 = Src[s * k + nx * j + nb_hi(i, nx)] - c;
                float w1 = Src[s * k + nx * j + nb_lo(i, nx)] - c;
                float n1 = Src[s * k + nx * nb_hi(j, ny) + i] - c;
                float s1 = Src[s * k + nx * nb_lo(j, ny) + i] - c;
                float u1 = 0.0f, d1 = 0.0f, sum;
                if (three) {
                    u1 = Src[s * nb_hi(k, nz) + nx * j + i] - c;
                    d1 = Src[s * nb_lo(k, nz) + nx * j + i] - c;
                }
                if (!linear) {
                    e1 = ndf_flux(e1, sg, penalty); w1 = ndf_flux(w1, sg, penalty);
                    n1 = ndf_flux(n1, sg, penalty); s1 = ndf_flux(s1, sg, penalty);
                    if (three) { u1 = ndf_flux(u1, sg, penalty); d1 = ndf_flux(d1, sg, penalty); }
                }
                sum = three ? (e1 + w1 + n1 + s1 + u1 + d1) : (e1 + w1 + n1 + s1);
                Dst[v] = c + tau * (lambda * sum - (c - F[v]));
            }
}

static float ndf_main(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                      int iterationsNumb, float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ,
                      int jacobi, const float *u_init)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ != 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz;
    float sg = (float)(sigmaPar / sqrt(2.0f));
    int linear = (sigmaPar == 0.0f), it;
    float *Uprev = NULL, *tmp = jacobi ? zalloc(n) : NULL;
    stop_state st = {0.0f, 0};
    if (!linear && (penaltytype < 1 || penaltytype > 5)) {
        free(tmp);
        return -1.0f;
    }
    if (epsil != 0.0f) Uprev = zalloc(n);
    copy_arr(u_init ? u_init : Input, Output, n);
    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        if (check) copy_arr(Output, Uprev, n);
        if (jacobi) {
            ndf_sweep(Input, Output, tmp, lambdaPar, sg, tau, penaltytype, linear, nx, ny, nz, 0);
            copy_arr(tmp, Output, n);
        } else {
            ndf_sweep(Input, Output, Output, lambdaPar, sg, tau, penaltytype, linear, nx, ny, nz, 1);
        }
        if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    free(Uprev); free(tmp);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

float port_Diffusion(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                     int iterationsNumb, float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ,
                     int jacobi)
{
    return ndf_main(Input, Output, infovector, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype, epsil, dimX,
                    dimY, dimZ, jacobi, NULL);
}

float port_Diffusion_init(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                          int iterationsNumb, float tau, int penaltytype, float epsil, int dimX, int dimY, int dimZ,
                          const float *u_init)
{
    return ndf_main(Input, Output, infovector, lambdaPar, sigmaPar, iterationsNumb, tau, penaltytype, epsil, dimX,
                    dimY, dimZ, 1, u_init);
}

/* ------------------------------------------------------------------ */
/* fourth-order anisotropic diffusion  (Diffus4th_order_core.c:44-265) */
/* ------------------------------------------------------------------ */
static void d4_weighted_laplacian(float *W, const float *U, float sg2, idx_t nx, idx_t ny, idx_t nz)
{
    idx_t i, j, k, s = nx * ny;
    const double eps = 1.0e-7;
#pragma omp parallel for private(i, j)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                idx_t ip = nb_hi(i, nx), im = nb_lo(i, nx), jp = nb_hi(j, ny), jm = nb_lo(j, ny);
                float gx, gy, gxx, gyy, gxy, gx2, gy2, xy2, den, vn, vo, c, c2;
                if (nz > 1) {
                    idx_t kp = nb_hi(k, nz), km = nb_lo(k, nz);
                    idx_t o = s * k, op = s * kp, om = s * km;
                    float gz, gz2, gzz, gxz, gyz, xz2, yz2;
                    gx = 0.5f * (U[o + nx * j + im] - U[o + nx * j + ip]); gx2 = gx * gx;
                    gy = 0.5f * (U[o + nx * jm + i] - U[o + nx * jp + i]); gy2 = gy * gy;
                    gz = 0.5f * (U[om + nx * j + i] - U[op + nx * j + i]); gz2 = gz * gz;
                    gxx = U[o + nx * j + im] + U[o + nx * j + ip] - 2 * U[v];
                    gyy = U[o + nx * jm + i] + U[o + nx * jp + i] - 2 * U[v];
                    gzz = U[om + nx * j + i] + U[op + nx * j + i] - 2 * U[v];
                    gxy = 0.25f * (U[o + nx * jm + im] + U[o + nx * jp + ip] - U[o + nx * jp + im] - U[o + nx * jm + ip]);
                    gxz = 0.25f * (U[om + nx * j + im] - U[om + nx * j + ip] - U[op + nx * j + im] + U[op + nx * j + ip]);
                    gyz = 0.25f * (U[om + nx * jm + i] - U[om + nx * jp + i] - U[op + nx * jm + i] + U[op + nx * jp + i]);
                    xy2 = 2.0f * gx * gy * gxy;
                    xz2 = 2.0f * gx * gz * gxz;
                    yz2 = 2.0f * gy * gz * gyz;
                    den = gx2 + gy2 + gz2;
                    {
                        float nn = gxx * gx2 + gyy * gy2 + gzz * gz2 + xy2 + xz2 + yz2;
                        float oo = (gy2 + gz2) * gxx + (gx2 + gz2) * gyy + (gx2 + gy2) * gzz - xy2 - xz2 - yz2;
                        if (den <= eps) { vn = (float)(nn / eps); vo = (float)(oo / eps); }
                        else { vn = nn / den; vo = oo / den; }
                    }
                } else {
                    gx = 0.5f * (U[nx * j + im] - U[nx * j + ip]); gx2 = gx * gx;
                    gy = 0.5f * (U[nx * jm + i] - U[nx * jp + i]); gy2 = gy * gy;
                    gxx = U[nx * j + im] + U[nx * j + ip] - 2 * U[v];
                    gyy = U[nx * jm + i] + U[nx * jp + i] - 2 * U[v];
                    gxy = 0.25f * (U[nx * jm + im] + U[nx * jp + ip] - U[nx * jp + im] - U[nx * jm + ip]);
                    xy2 = 2.0f * gx * gy * gxy;
                    den = gx2 + gy2;
                    {
                        float nn = gxx * gx2 + xy2 + gyy * gy2;
                        float oo = gxx * gy2 - xy2 + gyy * gx2;
                        if (den <= eps) { vn = (float)(nn / eps); vo = (float)(oo / eps); }
                        else { vn = nn / den; vo = oo / den; }
                    }
                }
                c = 1.0f / (1.0f + den / sg2);
                c2 = c * c;
                W[v] = c2 * vn + c * vo;
            }
}

static void d4_update(float *U, const float *F, const float *W, float lambda, float tau, idx_t nx, idx_t ny, idx_t nz)
{
    idx_t i, j, k, s = nx * ny;
#pragma omp parallel for private(i, j)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                float lx = W[s * k + nx * j + nb_lo(i, nx)] + W[s * k + nx * j + nb_hi(i, nx)] - 2 * W[v];
                float ly = W[s * k + nx * nb_lo(j, ny) + i] + W[s * k + nx * nb_hi(j, ny) + i] - 2 * W[v];
                if (nz > 1) {
                    float lz = W[s * nb_lo(k, nz) + nx * j + i] + W[s * nb_hi(k, nz) + nx * j + i] - 2 * W[v];
                    U[v] += tau * (-lambda * (lx + ly + lz) - (U[v] - F[v]));
                } else {
                    U[v] += tau * (-lambda * (lx + ly) - (U[v] - F[v]));
                }
            }
}

float port_Diffus4th(float *Input, float *Output, float *infovector, float lambdaPar, float sigmaPar,
                     int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ)
{
    if (dimZ < 1) dimZ = 1; /* a missing third axis means one slice */
    int three = dimZ != 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz;
    float sg2 = sigmaPar * sigmaPar;
    float *W = zalloc(n), *Uprev = NULL;
    stop_state st = {0.0f, 0};
    int it;
    if (epsil != 0.0f) Uprev = zalloc(n);
    copy_arr(Input, Output, n);
    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        if (check) copy_arr(Output, Uprev, n);
        d4_weighted_laplacian(W, Output, sg2, nx, ny, nz);
        d4_update(Output, Input, W, lambdaPar, tau, nx, ny, nz);
        if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    free(W); free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

/* number of OpenMP threads the port uses (1 when built without OpenMP) */
int port_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* LLT-ROF: fourth-order LLT + ROF-TV explicit flow                     */
/* (LLT_ROF_core.c:54-436)                                             */
/* ------------------------------------------------------------------ */
float port_LLT_ROF(float *Input, float *Output, float *infovector, float lambdaROF, float lambdaLLT,
                   int iterationsNumb, float tau, float epsil, int dimX, int dimY, int dimZ)
{
    if (dimZ < 1) dimZ = 1;
    idx_t nx = dimX, ny = dimY, nz = dimZ, n = nx * ny * nz, s = nx * ny;
    int three = nz > 1, it;
    float *R1 = zalloc(n), *R2 = zalloc(n), *R3 = zalloc(n);  /* ROF fluxes */
    float *L1 = zalloc(n), *L2 = zalloc(n), *L3 = zalloc(n);  /* normalised second derivatives */
    float *Uprev = NULL;
    stop_state st = {0.0f, 0};
    copy_arr(Input, Output, n);
    if (epsil != 0.0f) Uprev = zalloc(n);
    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        idx_t i, j, k;
        if (check) copy_arr(Output, Uprev, n);
        rof_fluxes(Output, R1, R2, R3, nx, ny, nz, 1.0e-12);
        /* der2D_LLT / der3D_LLT (LLT_ROF_core.c:131-188): dxx / (|dxx| + 1e-12),
         * the denominator formed in double and stored in a float */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float u = Output[v];
                    float dxx = Output[s * k + nx * j + nb_hi(i, nx)] - 2.0f * u + Output[s * k + nx * j + nb_lo(i, nx)];
                    float dyy = Output[s * k + nx * nb_hi(j, ny) + i] - 2.0f * u + Output[s * k + nx * nb_lo(j, ny) + i];
                    L1[v] = dxx / (float)(fabs(dxx) + 1.0e-12);
                    L2[v] = dyy / (float)(fabs(dyy) + 1.0e-12);
                    if (three) {
                        float dzz = Output[s * nb_hi(k, nz) + nx * j + i] - 2.0f * u + Output[s * nb_lo(k, nz) + nx * j + i];
                        L3[v] = dzz / (float)(fabs(dzz) + 1.0e-12);
                    }
                }
        /* Update2D_LLT_ROF / Update3D_LLT_ROF (LLT_ROF_core.c:377-436) */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    idx_t ip = nb_hi(i, nx), im = nb_lo(i, nx), jp = nb_hi(j, ny), jm = nb_lo(j, ny);
                    float dxx = L1[s * k + nx * j + ip] - 2.0f * L1[v] + L1[s * k + nx * j + im];
                    float dyy = L2[s * k + nx * jp + i] - 2.0f * L2[v] + L2[s * k + nx * jm + i];
                    float laplc, div;
                    if (three) {
                        idx_t kp = nb_hi(k, nz), km = nb_lo(k, nz);
                        float dzz = L3[s * kp + nx * j + i] - 2.0f * L3[v] + L3[s * km + nx * j + i];
                        laplc = dxx + dyy + dzz;
                        div = (R1[v] - R1[s * k + nx * jm + i]) + (R2[v] - R2[s * k + nx * j + im]) +
                              (R3[v] - R3[s * km + nx * j + i]);
                    } else {
                        laplc = dxx + dyy;
                        div = (R1[v] - R1[s * k + nx * jm + i]) + (R2[v] - R2[s * k + nx * j + im]);
                    }
                    Output[v] += tau * (lambdaROF * div - lambdaLLT * laplc - (Output[v] - Input[v]));
                }
        if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    free(R1); free(R2); free(R3); free(L1); free(L2); free(L3); free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

/* ------------------------------------------------------------------ */
/* FGP-dTV: FGP on the directional TV of a reference image             */
/* (FGP_dTV_core.c:46-380)                                             */
/* ------------------------------------------------------------------ */
float port_dTV_FGP(float *Input, float *InputRef, float *Output, float *infovector, float lambdaPar,
                   int iterationsNumb, float epsil, float eta, int methodTV, int nonneg, int dimX, int dimY,
                   int dimZ)
{
    if (dimZ < 1) dimZ = 1;
    int three = dimZ > 1;
    idx_t nx = dimX, ny = dimY, nz = three ? dimZ : 1, n = nx * ny * nz, s = nx * ny;
    float *P[3] = {0}, *Pold[3] = {0}, *R[3] = {0}, *B[3] = {0}, *Uprev = NULL;
    int c, na = three ? 3 : 2, it;
    float tk = 1.0f, tkp1 = 1.0f;
    float multip = three ? (1.0f / (26.0f * lambdaPar)) : (1.0f / (8.0f * lambdaPar));
    float eta_sq = eta * eta;
    stop_state st = {0.0f, 0};
    idx_t i, j, k;
    for (c = 0; c < na; c++) { P[c] = zalloc(n); Pold[c] = zalloc(n); R[c] = zalloc(n); B[c] = zalloc(n); }
    if (epsil != 0.0f) Uprev = zalloc(n);
    /* GradNorm_func2D/3D (:187-205, 273-300): eta-smoothed unit gradient of the
     * reference, forward differences with 0 beyond the last index */
#pragma omp parallel for private(i, j)
    for (k = 0; k < nz; k++)
        for (j = 0; j < ny; j++)
            for (i = 0; i < nx; i++) {
                idx_t v = s * k + nx * j + i;
                float b = InputRef[v];
                float gx = ((i == nx - 1) ? 0.0f : InputRef[v + 1]) - b;
                float gy = ((j == ny - 1) ? 0.0f : InputRef[v + nx]) - b;
                float magn;
                if (three) {
                    float gz = ((k == nz - 1) ? 0.0f : InputRef[v + s]) - b;
                    magn = gx * gx + gy * gy + gz * gz;
                    magn = (float)sqrt(magn + eta_sq);
                    B[2][v] = gz / magn;
                } else {
                    magn = gx * gx + gy * gy;
                    magn = (float)sqrt(magn + eta_sq);
                }
                B[0][v] = gx / magn;
                B[1][v] = gy / magn;
            }
    for (it = 0; it < iterationsNumb; it++) {
        int check = (epsil != 0.0f) && (it % 5 == 0);
        if (check) copy_arr(Output, Uprev, n);
        /* ProjectVect_func (:207-219, 302-317): R onto the complement of B */
#pragma omp parallel for
        for (i = 0; i < n; i++) {
            if (three) {
                float ip = R[0][i] * B[0][i] + R[1][i] * B[1][i] + R[2][i] * B[2][i];
                R[0][i] = R[0][i] - ip * B[0][i];
                R[1][i] = R[1][i] - ip * B[1][i];
                R[2][i] = R[2][i] - ip * B[2][i];
            } else {
                float ip = R[0][i] * B[0][i] + R[1][i] * B[1][i];
                R[0][i] = R[0][i] - ip * B[0][i];
                R[1][i] = R[1][i] - ip * B[1][i];
            }
        }
        /* Obj_dfunc (:221-234, 319-334): U = f - lambda div R, zero below index 0 */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float b1 = (i == 0) ? 0.0f : R[0][v - 1];
                    float b2 = (j == 0) ? 0.0f : R[1][v - nx];
                    if (three) {
                        float b3 = (k == 0) ? 0.0f : R[2][v - s];
                        Output[v] = Input[v] - lambdaPar * (R[0][v] + R[1][v] + R[2][v] - b1 - b2 - b3);
                    } else {
                        Output[v] = Input[v] - lambdaPar * (R[0][v] + R[1][v] - b1 - b2);
                    }
                }
        if (nonneg == 1) clamp_nonneg(Output, n);
        /* Grad_dfunc (:235-253, 335-363): gradient projected onto the complement of B */
#pragma omp parallel for private(i, j)
        for (k = 0; k < nz; k++)
            for (j = 0; j < ny; j++)
                for (i = 0; i < nx; i++) {
                    idx_t v = s * k + nx * j + i;
                    float g1 = (i == nx - 1) ? 0.0f : Output[v] - Output[v + 1];
                    float g2 = (j == ny - 1) ? 0.0f : Output[v] - Output[v + nx];
                    if (three) {
                        float g3 = (k == nz - 1) ? 0.0f : Output[v] - Output[v + s];
                        float ip = g1 * B[0][v] + g2 * B[1][v] + g3 * B[2][v];
                        g1 = g1 - ip * B[0][v];
                        g2 = g2 - ip * B[1][v];
                        g3 = g3 - ip * B[2][v];
                        P[2][v] = R[2][v] + multip * g3;
                    } else {
                        float ip = g1 * B[0][v] + g2 * B[1][v];
                        g1 = g1 - ip * B[0][v];
                        g2 = g2 - ip * B[1][v];
                    }
                    P[0][v] = R[0][v] + multip * g1;
                    P[1][v] = R[1][v] + multip * g2;
                }
        project_dual(P[0], P[1], three ? P[2] : NULL, methodTV, n);
        tkp1 = (float)((1.0f + sqrt(1.0f + 4.0f * tk * tk)) * 0.5f);
        {
            float m = (tk - 1.0f) / tkp1;
#pragma omp parallel for
            for (i = 0; i < n; i++)
                for (c = 0; c < na; c++) R[c][i] = P[c][i] + m * (P[c][i] - Pold[c][i]);
        }
        for (c = 0; c < na; c++) copy_arr(P[c], Pold[c], n);
        tk = tkp1;
        if (check && stop_check(&st, Output, Uprev, n, epsil)) break;
    }
    for (c = 0; c < na; c++) { free(P[c]); free(Pold[c]); free(R[c]); free(B[c]); }
    free(Uprev);
    infovector[0] = (float)it;
    infovector[1] = st.re;
    return 0;
}

/* ------------------------------------------------------------------ */
/* TV energy (utils.c:60-117): sequential FP32 sums in the reference's   */
/* loop order (2D: j, i; 3D: j, i, k)                                    */
/* ------------------------------------------------------------------ */
float port_TV_energy2D(float *U, float *U0, float *E_val, float lambda, int type, int dimX, int dimY)
{
    idx_t i, j, nx = dimX, ny = dimY;
    float eg = 0.0f, ed = 0.0f;
    for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++) {
            idx_t v = nx * j + i;
            idx_t i1 = (i == nx - 1) ? i : i + 1, j1 = (j == ny - 1) ? j : j + 1;
            float a = powf(U[nx * j1 + i] - U[v], 2);
            float b = powf(U[nx * j + i1] - U[v], 2);
            eg += 2.0f * lambda * sqrtf(a + b);
            ed += powf(U[v] - U0[v], 2);
        }
    if (type == 1) E_val[0] = eg + ed;
    if (type == 2) E_val[0] = eg;
    return E_val[0];
}

float port_TV_energy3D(float *U, float *U0, float *E_val, float lambda, int type, int dimX, int dimY, int dimZ)
{
    idx_t i, j, k, nx = dimX, ny = dimY, nz = dimZ, s = nx * ny;
    float eg = 0.0f, ed = 0.0f;
    for (j = 0; j < ny; j++)
        for (i = 0; i < nx; i++)
            for (k = 0; k < nz; k++) {
                idx_t v = s * k + nx * j + i;
                idx_t i1 = (i == nx - 1) ? i : i + 1, j1 = (j == ny - 1) ? j : j + 1, k1 = (k == nz - 1) ? k : k + 1;
                float a = powf(U[s * k + nx * j1 + i] - U[v], 2);
                float b = powf(U[s * k + nx * j + i1] - U[v], 2);
                float c = powf(U[s * k1 + nx * j + i] - U[v], 2);
                eg += 2.0f * lambda * sqrtf(a + b + c);
                ed += powf(U[v] - U0[v], 2);
            }
    if (type == 1) E_val[0] = eg + ed;
    if (type == 2) E_val[0] = eg;
    return E_val[0];
}
