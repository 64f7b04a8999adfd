// lbm_collide.cuh -- the per-cell collision operators shared by the step,
// band and fused IBM kernels.
#pragma once
#include "lbm_device.cuh"

namespace lbmk {

// 1 / (1 + drho) without the rounding of 1 + drho: with s = fl(1 + drho) the
// exact sum is s + e, e = drho - (s - 1) (Fast2Sum), and 1/(s + e) is taken to
// first order in e.  drho ~ 1e-3 loses ~1e-7 relative in fl(1 + drho); over
// thousands of steps that bias dominates the FP32 velocity error.
__device__ __forceinline__ float inv_one_plus(float drho) {
    const float s = 1.0f + drho;
    const float e = drho - (s - 1.0f);
    const float inv = __frcp_rn(s);  // correctly rounded, as 1.0f / s
    return inv - inv * inv * e;
}

// BGK + Guo collision on shifted populations (f~ = f - w), FP32:
//   f~* = (1 - omega) f~ + omega (feq - w) + S,
//   feq - w = w (drho + rho P3(u)) with the third-order P3 of Calc_feq
//   (lbm.cpp:628-633), S = (1 - omega/2) w (3 c.F + 9 (c.F)(c.u) - 3 F.u)
//   (lbm.cpp:101-102).
// Links come in opposite pairs (l, l+1) for odd l (LBM.h:551), so
// P3 = E(cu) +/- O(cu) with E = 4.5 cu^2 - 1.5 u^2 and
// O = cu (3 + 4.5 (cu^2 - u^2)), and likewise for S: the pair shares one
// evaluation of each part.  Per weight class the factors omega w rho and
// omega w (drho - 1.5 rho u^2) are formed once, so a pair costs a square, one
// fused multiply-add for the even part, three operations for the odd part
// and two fused multiply-adds per link.  drho enters additively, never
// through fl(1 + drho).
__device__ __forceinline__ void collide_flow(float f[Q], float drho, float ux, float uy, float uz, float Fx,
                                             float Fy, float Fz, bool forced, float omega) {
    const float usq = ux * ux + uy * uy + uz * uz;
    const float c1 = 1.0f - omega;
    const float rho = 1.0f + drho;
    const float orho = omega * rho;
    const float odrho = omega * drho;
    const float m15 = -1.5f * usq;
    const float t3 = fmaf(-4.5f, usq, 3.0f);
    // class 0 (rest), 1 (axis), 2 (diagonal)
    const float k0 = orho * wf(0), k1 = orho * wf(1), k2 = orho * wf(7);
    const float b0 = fmaf(k0, m15, odrho * wf(0));
    const float b1 = fmaf(k1, m15, odrho * wf(1));
    const float b2 = fmaf(k2, m15, odrho * wf(7));
    const float h1 = 4.5f * k1, h2 = 4.5f * k2;
    const float gs = 1.0f - 0.5f * omega;
    const float Fu = Fx * ux + Fy * uy + Fz * uz;
    f[0] = fmaf(c1, f[0], b0);
    if (forced) f[0] += gs * wf(0) * (-3.0f * Fu);
#pragma unroll
    for (int l = 1; l < Q; l += 2) {
        const bool diag = (l >= 7);
        const float k = diag ? k2 : k1, bb = diag ? b2 : b1, hh = diag ? h2 : h1;
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float cu2 = cu * cu;
        const float ev = fmaf(hh, cu2, bb);              // omega w (drho + rho E)
        const float od = (k * cu) * fmaf(4.5f, cu2, t3);  // omega w rho O
        float a = fmaf(c1, f[l], ev + od);
        float b = fmaf(c1, f[l + 1], ev - od);
        if (forced) {
            const float cF = cx(l) * Fx + cy(l) * Fy + cz(l) * Fz;
            const float gw = gs * wf(l);
            const float e = gw * fmaf(9.0f * cF, cu, -3.0f * Fu);
            const float o = gw * (3.0f * cF);
            a += e + o;
            b += e - o;
        }
        f[l] = a;
        f[l + 1] = b;
    }
}

// Moments of shifted populations, summed by opposite pairs:
// drho = sum f~, j = sum c f~ (sum w = 1, sum w c = 0).
__device__ __forceinline__ void moments_pairs(const float f[Q], float &drho, float &jx, float &jy, float &jz) {
    float r = f[0], x = 0.0f, y = 0.0f, z = 0.0f;
#pragma unroll
    for (int l = 1; l < Q; l += 2) {
        const float s = f[l] + f[l + 1], d = f[l] - f[l + 1];
        r += s;
        if (cx(l) != 0) x += cx(l) * d;
        if (cy(l) != 0) y += cy(l) * d;
        if (cz(l) != 0) z += cz(l) * d;
    }
    drho = r;
    jx = x;
    jy = y;
    jz = z;
}

// D3Q7 BGK with source: g* = g - omega_t (g - w T (1 + 4 c.u)) + (1 - omega_t/2) w Qh.
__device__ __forceinline__ void collide_heat(float g[QT], float T, float ux, float uy, float uz, float Qh,
                                             float omega_t) {
    const float gsrc = 1.0f - 0.5f * omega_t;
#pragma unroll
    for (int l = 0; l < QT; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float geq = wtf(l) * T * (1.0f + 4.0f * cu);
        g[l] = g[l] - omega_t * (g[l] - geq) + gsrc * wtf(l) * Qh;
    }
}

// Fused step.  gather = 0 on the first step (A then holds the initial
// pre-collision populations in place); export_only = 1 computes and writes
// the moments of the gathered state without colliding or storing.
}  // namespace lbmk
