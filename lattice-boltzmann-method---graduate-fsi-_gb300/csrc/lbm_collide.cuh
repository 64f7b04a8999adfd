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
//   feq - w = w (drho + (1 + drho) P3(u)) with the third-order P3 of Calc_feq
//   (lbm.cpp:628-633), S = (1 - omega/2) w (3 c.F + 9 (c.F)(c.u) - 3 F.u)
//   (lbm.cpp:101-102).
// Links come in opposite pairs (l, l+1) for odd l (LBM.h:551), so
// P3 = E(cu) +/- O(cu) with E = 4.5 cu^2 - 1.5 u^2 and
// O = cu (3 + 4.5 (cu^2 - u^2)), and likewise for S: the pair shares one
// evaluation of each part.
__device__ __forceinline__ void collide_flow(float f[Q], float drho, float ux, float uy, float uz, float Fx,
                                             float Fy, float Fz, bool forced, float omega) {
    const float usq = ux * ux + uy * uy + uz * uz;
    const float c1 = 1.0f - omega;
    const float gs = 1.0f - 0.5f * omega;
    const float Fu = Fx * ux + Fy * uy + Fz * uz;
    {
        const float p = -1.5f * usq;
        f[0] = c1 * f[0] + omega * wf(0) * (drho + p + drho * p);
        if (forced) f[0] += gs * wf(0) * (-3.0f * Fu);
    }
#pragma unroll
    for (int l = 1; l < Q; l += 2) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float cu2 = cu * cu;
        const float ev = 4.5f * cu2 - 1.5f * usq;
        const float od = cu * (3.0f + 4.5f * (cu2 - usq));
        // (1 + drho) x without forming 1 + drho
        const float be = drho + ev + drho * ev;
        const float bo = od + drho * od;
        const float ow = omega * wf(l);
        float a = c1 * f[l] + ow * (be + bo);
        float b = c1 * f[l + 1] + ow * (be - bo);
        if (forced) {
            const float cF = cx(l) * Fx + cy(l) * Fy + cz(l) * Fz;
            const float e = 9.0f * cF * cu - 3.0f * Fu;
            const float o = 3.0f * cF;
            const float gw = gs * wf(l);
            a += gw * (e + o);
            b += gw * (e - o);
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
