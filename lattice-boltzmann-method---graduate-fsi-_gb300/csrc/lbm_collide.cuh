// lbm_collide.cuh -- the per-cell collision operators shared by the step,
// band and fused IBM kernels.
//
// The arithmetic is written once for one cell (F = float) and for two
// neighbouring cells at a time (F = float2, the packed FP32 pair
// instructions of sm_100+: one instruction updates both cells).  Every
// operation is rounded explicitly (fma/mul/add with round-to-nearest, never
// left to contraction), so a cell gets bit-identical results from either
// form and from every kernel that uses them.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "lbm_device.cuh"

namespace lbmk {

template <class F>
struct Ar;
template <>
struct Ar<float> {
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    // a - b, rounded once (as fma(b, -1, a))
    static __device__ __forceinline__ float sub(float a, float b) { return __fmaf_rn(b, -1.0f, a); }
    static __device__ __forceinline__ float splat(float s) { return s; }
};
template <>
struct Ar<float2> {
    static __device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
    static __device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ float2 sub(float2 a, float2 b) {
        return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
    }
    static __device__ __forceinline__ float2 splat(float s) { return make_float2(s, s); }
};

// 1 / (1 + drho) without the rounding of 1 + drho: with s = fl(1 + drho) the
// exact sum is s + e, e = drho - (s - 1) (Fast2Sum), and 1/(s + e) is taken to
// first order in e.
__device__ __forceinline__ float inv_one_plus(float drho) {
    const float s = __fadd_rn(1.0f, drho);
    const float e = __fadd_rn(drho, -__fadd_rn(s, -1.0f));
    const float inv = __frcp_rn(s);  // correctly rounded, as 1.0f / s
    return __fmaf_rn(-__fmul_rn(inv, inv), e, inv);
}
__device__ __forceinline__ float2 inv_one_plus(float2 drho) {
    return make_float2(inv_one_plus(drho.x), inv_one_plus(drho.y));
}

// c . v for a D3Q19 link with components in {-1, 0, 1}: sums and differences
// only (one rounding for a two-term sum).
template <class F, int L>
__device__ __forceinline__ F cdot(F vx, F vy, F vz) {
    using A = Ar<F>;
    constexpr int a = cx(L), b = cy(L), c = cz(L);
    if constexpr (a != 0 && b != 0) return a > 0 ? (b > 0 ? A::add(vx, vy) : A::sub(vx, vy)) : A::sub(vy, vx);
    else if constexpr (a != 0 && c != 0) return a > 0 ? (c > 0 ? A::add(vx, vz) : A::sub(vx, vz)) : A::sub(vz, vx);
    else if constexpr (b != 0 && c != 0) return b > 0 ? (c > 0 ? A::add(vy, vz) : A::sub(vy, vz)) : A::sub(vz, vy);
    else if constexpr (a != 0) return a > 0 ? vx : A::sub(A::splat(0.0f), vx);
    else if constexpr (b != 0) return b > 0 ? vy : A::sub(A::splat(0.0f), vy);
    else if constexpr (c != 0) return c > 0 ? vz : A::sub(A::splat(0.0f), vz);
    else return A::splat(0.0f);
}

// fn(integral_constant<l>) for the odd links l = L, L+2, ... < Q.
template <int L, class Fn>
__device__ __forceinline__ void for_pairs(Fn &&fn) {
    if constexpr (L < Q) {
        fn(std::integral_constant<int, L>{});
        for_pairs<L + 2>(fn);
    }
}

// Moments of shifted populations, summed by opposite pairs (l, l+1), l odd
// (LBM.h:551): drho = sum f~, j = sum c f~ (sum w = 1, sum w c = 0).
template <class F>
__device__ __forceinline__ void moments_pairs(const F f[Q], F &drho, F &jx, F &jy, F &jz) {
    using A = Ar<F>;
    F r = f[0], x = A::splat(0.0f), y = A::splat(0.0f), z = A::splat(0.0f);
    for_pairs<1>([&](auto li) {
        constexpr int l = decltype(li)::value;
        const F s = A::add(f[l], f[l + 1]), d = A::sub(f[l], f[l + 1]);
        r = A::add(r, s);
        if constexpr (cx(l) > 0) x = A::add(x, d);
        if constexpr (cx(l) < 0) x = A::sub(x, d);
        if constexpr (cy(l) > 0) y = A::add(y, d);
        if constexpr (cy(l) < 0) y = A::sub(y, d);
        if constexpr (cz(l) > 0) z = A::add(z, d);
        if constexpr (cz(l) < 0) z = A::sub(z, d);
    });
    drho = r;
    jx = x;
    jy = y;
    jz = z;
}

// BGK + Guo collision on shifted populations (f~ = f - w), FP32:
//   f~* = (1 - omega) f~ + omega (feq - w) + S,
//   feq - w = w (drho + rho P3(u)) with the third-order P3 of Calc_feq
//   (lbm.cpp:628-633), S = (1 - omega/2) w (3 c.F + 9 (c.F)(c.u) - 3 F.u)
//   (lbm.cpp:101-102).
// Links come in opposite pairs (l, l+1), so P3 = E(cu) +/- O(cu) with
// E = 4.5 cu^2 - 1.5 u^2 and O = cu (3 + 4.5 (cu^2 - u^2)), and likewise for
// S: the pair shares one evaluation of each part.  Per weight class the
// factors omega w rho and omega w (drho - 1.5 rho u^2) are formed once.  drho
// enters additively, never through fl(1 + drho).
template <class F, bool FORCED>
__device__ __forceinline__ void collide_flow(F f[Q], F drho, F ux, F uy, F uz, F Fx, F Fy, F Fz, float omega) {
    using A = Ar<F>;
    const F usq = A::fma(uz, uz, A::fma(uy, uy, A::mul(ux, ux)));
    const F c1 = A::splat(1.0f - omega);
    const F orho = A::mul(A::splat(omega), A::add(A::splat(1.0f), drho));
    const F odrho = A::mul(A::splat(omega), drho);
    const F m15 = A::mul(A::splat(-1.5f), usq);
    const F t3 = A::fma(A::splat(-4.5f), usq, A::splat(3.0f));
    // class 0 (rest), 1 (axis), 2 (diagonal)
    const F k0 = A::mul(orho, A::splat(wf(0))), k1 = A::mul(orho, A::splat(wf(1))), k2 = A::mul(orho, A::splat(wf(7)));
    const F b0 = A::fma(k0, m15, A::mul(odrho, A::splat(wf(0))));
    const F b1 = A::fma(k1, m15, A::mul(odrho, A::splat(wf(1))));
    const F b2 = A::fma(k2, m15, A::mul(odrho, A::splat(wf(7))));
    const F h1 = A::mul(A::splat(4.5f), k1), h2 = A::mul(A::splat(4.5f), k2);
    const float gs = 1.0f - 0.5f * omega;
    F m3Fu = A::splat(0.0f);
    if constexpr (FORCED) m3Fu = A::mul(A::splat(-3.0f), A::fma(Fz, uz, A::fma(Fy, uy, A::mul(Fx, ux))));
    f[0] = A::fma(c1, f[0], b0);
    if constexpr (FORCED) f[0] = A::fma(A::splat(gs * wf(0)), m3Fu, f[0]);
    for_pairs<1>([&](auto li) {
        constexpr int l = decltype(li)::value;
        constexpr bool diag = (l >= 7);
        const F k = diag ? k2 : k1, bb = diag ? b2 : b1, hh = diag ? h2 : h1;
        const F cu = cdot<F, l>(ux, uy, uz);
        const F cu2 = A::mul(cu, cu);
        const F ev = A::fma(hh, cu2, bb);                                      // omega w (drho + rho E)
        const F od = A::mul(A::mul(k, cu), A::fma(A::splat(4.5f), cu2, t3));  // omega w rho O
        F a = A::fma(c1, f[l], A::add(ev, od));
        F b = A::fma(c1, f[l + 1], A::sub(ev, od));
        if constexpr (FORCED) {
            const F cF = cdot<F, l>(Fx, Fy, Fz);
            const F gw = A::splat(gs * wf(l));
            const F e = A::mul(gw, A::fma(A::mul(A::splat(9.0f), cF), cu, m3Fu));
            const F o = A::mul(gw, A::mul(A::splat(3.0f), cF));
            a = A::add(a, A::add(e, o));
            b = A::add(b, A::sub(e, o));
        }
        f[l] = a;
        f[l + 1] = b;
    });
}

// The one-cell form with a run-time forcing switch (band and batch kernels).
__device__ __forceinline__ void collide_flow(float f[Q], float drho, float ux, float uy, float uz, float Fx, float Fy,
                                             float Fz, bool forced, float omega) {
    if (forced) collide_flow<float, true>(f, drho, ux, uy, uz, Fx, Fy, Fz, omega);
    else collide_flow<float, false>(f, drho, ux, uy, uz, Fx, Fy, Fz, omega);
}

// D3Q7 BGK with source: g* = g - omega_t (g - w T (1 + 4 c.u)) + (1 - omega_t/2) w Qh.
// Links 2a+1 and 2a+2 are +e_a and -e_a.
template <class F, bool SOURCE>
__device__ __forceinline__ void collide_heat(F g[QT], F T, F ux, F uy, F uz, F Qh, float omega_t) {
    using A = Ar<F>;
    const F nom = A::splat(-omega_t);
    const float gsrc = 1.0f - 0.5f * omega_t;
    const F w0T = A::mul(A::splat(wtf(0)), T), w1T = A::mul(A::splat(wtf(1)), T);
    g[0] = A::fma(nom, A::sub(g[0], w0T), g[0]);
    if constexpr (SOURCE) g[0] = A::fma(A::splat(gsrc * wtf(0)), Qh, g[0]);
    const F u[3] = {ux, uy, uz};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const F t4 = A::mul(A::splat(4.0f), u[a]);
        const F gp = A::mul(w1T, A::add(A::splat(1.0f), t4));
        const F gm = A::mul(w1T, A::sub(A::splat(1.0f), t4));
        F p = A::fma(nom, A::sub(g[2 * a + 1], gp), g[2 * a + 1]);
        F m = A::fma(nom, A::sub(g[2 * a + 2], gm), g[2 * a + 2]);
        if constexpr (SOURCE) {
            p = A::fma(A::splat(gsrc * wtf(1)), Qh, p);
            m = A::fma(A::splat(gsrc * wtf(1)), Qh, m);
        }
        g[2 * a + 1] = p;
        g[2 * a + 2] = m;
    }
}

// Temperature sum g (lbm.cpp:778-792, D3Q7), in a fixed order.
template <class F>
__device__ __forceinline__ F heat_sum(const F g[QT]) {
    using A = Ar<F>;
    F t = g[0];
#pragma unroll
    for (int l = 1; l < QT; l++) t = A::add(t, g[l]);
    return t;
}

}  // namespace lbmk
