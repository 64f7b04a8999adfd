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
    const float inv = 1.0f / s;
    return inv - inv * inv * e;
}

// BGK + Guo collision on shifted populations (f~ = f - w), FP32:
//   f~* = (1 - omega) f~ + omega (feq - w) + S,
//   feq - w = w (drho + (1 + drho) P3(u)) with the third-order P3 of Calc_feq
//   (lbm.cpp:628-633), S = (1 - omega/2) w (3 c.F + 9 (c.F)(c.u) - 3 F.u)
//   (lbm.cpp:101-102).
__device__ __forceinline__ void collide_flow(float f[Q], float drho, float ux, float uy, float uz, float Fx,
                                             float Fy, float Fz, bool forced, float omega) {
    const float usq = ux * ux + uy * uy + uz * uz;
    const float c1 = 1.0f - omega;
    const float gs = 1.0f - 0.5f * omega;
    const float Fu = Fx * ux + Fy * uy + Fz * uz;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float p3 = cu * (3.0f + 4.5f * cu + 4.5f * cu * cu - 4.5f * usq) - 1.5f * usq;
        // w (rho (1 + P3) - 1) = w (drho + P3 + drho P3), without forming 1 + drho
        float out = c1 * f[l] + omega * wf(l) * (drho + p3 + drho * p3);
        if (forced) {
            const float cF = cx(l) * Fx + cy(l) * Fy + cz(l) * Fz;
            out += gs * wf(l) * (3.0f * cF + 9.0f * cF * cu - 3.0f * Fu);
        }
        f[l] = out;
    }
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
