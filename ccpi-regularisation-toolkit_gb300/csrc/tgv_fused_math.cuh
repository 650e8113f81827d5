// Per-voxel arithmetic of one fused TGV iteration (3D), shared by the
// thread-loading pass (tgv_fused.cu) and the pass whose inputs are staged by
// tensor copies (tgv_fused_tma.cu), so both give the same iterates bit for
// bit.  The expressions are those of the two half-iteration passes
// (tgv_tiled.cu), which follow TGV_core.c:351-568.
#pragma once

namespace cilreg {

// new dual variables of one voxel: P (3 components) and Q (6, symmetric)
struct TgvDual {
    float p1, p2, p3, q1, q2, q3, q4, q5, q6;
};

// the new V (3 components) of one voxel
struct TgvNewV {
    float v1, v2, v3;
};

__device__ __forceinline__ float tgv_bwd(float x, float xprev, bool first, bool last) {
    return first ? x : (last ? -xprev : x - xprev);
}

// Dual half at one voxel (DualP_3D + ProjP_3D, DualQ_3D + ProjQ_3D,
// TGV_core.c:351-446): forward differences of U and V, the ascent step from
// the old P, Q (pq: P1..P3, Q1..Q6) and the projections onto the alpha1 and
// alpha0 balls.  u, v1..v3 are the voxel's U, V; xn(c), yn(c), zn(c) return
// component c (0: U, 1..3: V1..V3) at its forward neighbours, and are not
// called on the last voxel of that axis (xe, ye, ze).
template <class XN, class YN, class ZN>
__device__ __forceinline__ TgvDual tgv_dual_voxel(float u, float v1, float v2, float v3, XN xn, YN yn, ZN zn,
                                                  const float pq[9], bool xe, bool ye, bool ze, float sigma,
                                                  float alpha1, float alpha0) {
    TgvDual n;
    float p1 = pq[0] + (xe ? sigma * (-v1) : sigma * ((xn(0) - u) - v1));
    float p2 = pq[1] + (ye ? sigma * (-v2) : sigma * ((yn(0) - u) - v2));
    float p3 = pq[2] + (ze ? sigma * (-v3) : sigma * ((zn(0) - u) - v3));
    const float gp = sqrtf(p1 * p1 + p2 * p2 + p3 * p3) / alpha1;
    if (gp > 1.0f) {
        const float ig = __frcp_rn(gp);
        p1 *= ig;
        p2 *= ig;
        p3 *= ig;
    }
    float q1 = 0.f, q11 = 0.f, q33 = 0.f, q2 = 0.f, q22 = 0.f, q55 = 0.f, q3 = 0.f, q44 = 0.f, q66 = 0.f;
    if (!xe) {
        q1 = xn(1) - v1;
        q11 = xn(2) - v2;
        q33 = xn(3) - v3;
    }
    if (!ye) {
        q2 = yn(2) - v2;
        q22 = yn(1) - v1;
        q55 = yn(3) - v3;
    }
    if (!ze) {
        q3 = zn(3) - v3;
        q44 = zn(1) - v1;
        q66 = zn(2) - v2;
    }
    float Q1 = pq[3] + sigma * q1;
    float Q2 = pq[4] + sigma * q2;
    float Q3 = pq[5] + sigma * q3;
    float Q4 = pq[6] + sigma * (0.5f * (q11 + q22));
    float Q5 = pq[7] + sigma * (0.5f * (q33 + q44));
    float Q6 = pq[8] + sigma * (0.5f * (q55 + q66));
    float g = sqrtf(Q1 * Q1 + Q2 * Q2 + Q3 * Q3 + 2.0f * Q4 * Q4 + 2.0f * Q5 * Q5 + 2.0f * Q6 * Q6);
    g = g / alpha0;
    if (g > 1.0f) {
        const float ig = __frcp_rn(g);
        Q1 *= ig;
        Q2 *= ig;
        Q3 *= ig;
        Q4 *= ig;
        Q5 *= ig;
        Q6 *= ig;
    }
    n.p1 = p1;
    n.p2 = p2;
    n.p3 = p3;
    n.q1 = Q1;
    n.q2 = Q2;
    n.q3 = Q3;
    n.q4 = Q4;
    n.q5 = Q5;
    n.q6 = Q6;
    return n;
}

// Primal half at one voxel (DivProjP_3D + newU3D, UpdV_3D + newV,
// TGV_core.c:448-568), from the voxel's new dual n and the components of its
// backward neighbours that the divergences need.  U: the extrapolated new U
// (2 U_new - U) from the old U cu, the data u0 and P1 at x-1, P2 at y-1, P3
// at z-1.
__device__ __forceinline__ float tgv_primal_u(const TgvDual& n, float xp1, float yp2, float zp3, bool xf, bool xe,
                                              bool yf, bool ye, bool zf, bool zl, float cu, float u0, float lam,
                                              float tau, float ilt) {
    float dv = tgv_bwd(n.p1, xp1, xf, xe) + tgv_bwd(n.p2, yp2, yf, ye);
    dv = dv + tgv_bwd(n.p3, zp3, zf, zl);
    const float un = (lam * (cu + tau * dv) + tau * u0) * ilt;
    return 2.0f * un - cu;
}

// V: the extrapolated new V from the old V (v1..v3) and Q1, Q4, Q5 at x-1;
// Q2, Q4, Q6 at y-1; Q3, Q5, Q6 at z-1.
__device__ __forceinline__ TgvNewV tgv_primal_v(const TgvDual& n, float xq1, float xq4, float xq5, float yq2,
                                                float yq4, float yq6, float zq3, float zq5, float zq6, bool xf,
                                                bool xe, bool yf, bool ye, bool zf, bool zl, float v1, float v2,
                                                float v3, float tau) {
    TgvNewV o;
    const float q1 = tgv_bwd(n.q1, xq1, xf, xe), q4x = tgv_bwd(n.q4, xq4, xf, xe), q5x = tgv_bwd(n.q5, xq5, xf, xe);
    const float q2 = tgv_bwd(n.q2, yq2, yf, ye), q4y = tgv_bwd(n.q4, yq4, yf, ye), q6y = tgv_bwd(n.q6, yq6, yf, ye);
    const float q6z = tgv_bwd(n.q6, zq6, zf, zl), q5z = tgv_bwd(n.q5, zq5, zf, zl), q3 = tgv_bwd(n.q3, zq3, zf, zl);
    const float d1 = q1 + q4y + q5z, d2 = q4x + q2 + q6z, d3 = q5x + q6y + q3;
    o.v1 = 2.0f * (v1 + tau * (n.p1 + d1)) - v1;
    o.v2 = 2.0f * (v2 + tau * (n.p2 + d2)) - v2;
    o.v3 = 2.0f * (v3 + tau * (n.p3 + d3)) - v3;
    return o;
}

}  // namespace cilreg
