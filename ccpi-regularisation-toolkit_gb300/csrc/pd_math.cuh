// Per-voxel PD-TV arithmetic rounded exactly as the reference C code
// (PD_TV_core.c:212-252, utils.c:180-213): every multiply and add rounded
// separately (no contraction into fused multiply-adds), the isotropic
// projection with an IEEE square root and division, and the primal update's
// division by the double (1.0 + lt) reproduced in FP32.
//
// PD's extrapolation (theta = 1) lets per-voxel rounding differences grow
// over hundreds of iterations; with this rounding the iterates follow the
// reference's to within its own double rounding (a float numerator divided in
// double and stored as float).
#pragma once

#include <cuda_runtime.h>

#include "common.cuh"

namespace cilreg {

// The reference's  (float)((double)num / D)  with D = 1.0 + lt a double:
// D = hi + lo (hi its float rounding, lo the float rounding of the rest) and
// rcp the float rounding of 1/D.  q = num rcp is within an ulp or so of the
// quotient; r = num - q hi is exact in one fused multiply-add (a remainder
// of a near-quotient), r - q lo brings in the low part of D (its own rounding
// error is far below an ulp of q), and q + r rcp is the rounded quotient.
// Checked against the double division on 10^8 random numerators for several
// lt (no difference).
struct DoubleDivisor {
    float hi, lo, rcp;
};

inline DoubleDivisor make_double_divisor(double D) {
    DoubleDivisor v;
    v.hi = (float)D;
    v.lo = (float)(D - (double)v.hi);
    v.rcp = (float)(1.0 / D);
    return v;
}

__device__ __forceinline__ float div_by_double(float num, const DoubleDivisor& D) {
    const float q = __fmul_rn(num, D.rcp);
    float r = __fmaf_rn(-q, D.hi, num);
    r = __fsub_rn(r, __fmul_rn(q, D.lo));
    return __fmaf_rn(r, D.rcp, q);
}

// P + sigma (Ue[+1] - Ue)  (PD_TV_core.c:222-227)
__device__ __forceinline__ float pd_dual(float p, float sigma, float u_hi, float u) {
    return __fadd_rn(p, __fmul_rn(sigma, __fsub_rn(u_hi, u)));
}

// isotropic projection: denom = P1^2 + P2^2 (+ P3^2); if denom > 1 every
// component times 1/sqrtf(denom)  (utils.c:185-195)
template <bool THREE>
__device__ __forceinline__ void pd_project_iso(float& p1, float& p2, float& p3) {
    float den = __fadd_rn(__fmul_rn(p1, p1), __fmul_rn(p2, p2));
    if (THREE) den = __fadd_rn(den, __fmul_rn(p3, p3));
    if (den > 1.0f) {
        const float s = __fdiv_rn(1.0f, __fsqrt_rn(den));
        p1 = __fmul_rn(p1, s);
        p2 = __fmul_rn(p2, s);
        if (THREE) p3 = __fmul_rn(p3, s);
    }
}

// anisotropic projection: each component over max(|P_c|, 1)  (utils.c:198-210)
__device__ __forceinline__ float pd_project_aniso(float p) { return unit_clip(p); }

// U = (U - tau div + lt f) / (1.0 + lt)  (PD_TV_core.c:249)
__device__ __forceinline__ float pd_primal(float u, float tau, float dv, float lt, float f, const DoubleDivisor& D) {
    const float num = __fadd_rn(__fsub_rn(u, __fmul_rn(tau, dv)), __fmul_rn(lt, f));
    return div_by_double(num, D);
}

// getX: U + theta (U - U_old)  (PD_TV_core.c:197-205)
__device__ __forceinline__ float pd_extrapolate(float unew, float theta, float uold) {
    return __fadd_rn(unew, __fmul_rn(theta, __fsub_rn(unew, uold)));
}

}  // namespace cilreg
