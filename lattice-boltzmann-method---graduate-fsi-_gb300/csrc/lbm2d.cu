// lbm2d.cu -- the reference's two-dimensional build (#define D2Q9) on the
// device: D2Q9 BGK with Guo forcing and pull streaming, and the 2D immersed
// boundary of IBLBM (lbm.cpp:1135-1416) with the reference's own options.
//
// One reference iteration (IBLBM -> Collision -> Streaming) is two launches:
//   k_step2d  gather (= Streaming of the previous step, lbm.cpp:182-296),
//             moments, BGK + Guo collision (lbm.cpp:60-119); cells inside the
//             IBM box store their pre-collision populations and unforced
//             moments instead.
//   k_ibm2d   one thread block: the whole IBM pass on the box -- marker
//             stencils, the implicit multi-direct forcing (lbm.cpp:1259-1390)
//             or the explicit direct forcing (lbm.cpp:1171-1258), the added
//             mass (lbm.cpp:1392-1398), the collision of the box cells, and
//             the body kinematics of the next step (lbm.cpp:1140-1167).
// A box of (2D+2)^2 nodes and a few hundred markers is far too little work
// for more than one block; one block runs the m_max iterations with block
// barriers only, its working fields staying in L2.
//
// Spreading is node-centred: each box node sums the forces of the markers
// whose stencil covers it, in ascending marker order, through lists built
// from the stencils (once for a fixed body, every step for a moving one) --
// the reference's order of summation (lbm.cpp:1336-1344), with no atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "lbm2d.cuh"
#include "lbm_device.cuh"
#include "lbm_handle.h"

namespace l2d {

using lbmk::St;

constexpr int kIbmBlock = 1024;
constexpr double kRefPi = 3.14159265;  // the reference's truncated PI (LBM.h:74)

// ---------------------------------------------------------------------------
// Collide-stream
// ---------------------------------------------------------------------------
// One status update per warp from the lanes still running (the step
// kernels let lanes past the grid edge leave early): a diverged solve would
// otherwise send an atomic from every cell.
__device__ __forceinline__ void status_once(uint32_t *status, uint32_t bit, bool bad) {
    const unsigned am = __activemask();
    const unsigned b = __ballot_sync(am, bad);
    if (b && (threadIdx.x & 31) == (unsigned)(__ffs(am) - 1)) lbmk::raise_status(status, bit);
}

template <class T>
__device__ __forceinline__ float pull_link2(const T *__restrict__ A, int l, int x, int y, long long cell,
                                            const Class2 &ce, const Params2 &P) {
    if ((ce.bb >> l) & 1u) return St<T>::ld(A + opp9(l) * P.S + cell) + ce.val[l];
    if ((ce.eq >> l) & 1u) return ce.val[l];
    int sx = x - cx9(l), sy = y - cy9(l);
    if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
    if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
    if ((ce.zg >> l) & 1u) {
        sx = min(max(sx, 0), P.nx - 1);
        sy = min(max(sy, 0), P.ny - 1);
    }
    return St<T>::ld(A + l * P.S + sx + (long long)P.nx * sy);
}

// BGK + Guo on shifted populations (ConvLBM, lbm.cpp:91-118, with the D2Q9
// tables; cs^2 = 1/3): f~* = f~ (1 - w) + w (feq - w_l) + S.
__device__ __forceinline__ void collide9(float f[Q9], float drho, float ux, float uy, float Fx, float Fy,
                                         float omega, bool forced) {
    const float rho = 1.0f + drho;
    const float usq = ux * ux + uy * uy;
    const float c1 = 1.0f - 0.5f * omega;
    const float Fu = Fx * ux + Fy * uy;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        const float cu = (float)cx9(l) * ux + (float)cy9(l) * uy;
        const float poly = 3.0f * cu + 4.5f * cu * cu - 1.5f * usq + 4.5f * cu * cu * cu - 4.5f * cu * usq;
        const float feq_s = w9f(l) * (drho + rho * poly);
        float v = f[l] * (1.0f - omega) + omega * feq_s;
        if (forced) {
            const float Fc = (float)cx9(l) * Fx + (float)cy9(l) * Fy;
            v += c1 * w9f(l) * (3.0f * Fc + 9.0f * Fc * cu - 3.0f * Fu);
        }
        f[l] = v;
    }
}

// With SOLID, interior solid cells (staircase bodies at rest) keep their
// populations (the reference never collides or streams them, so they hold
// their set-up equilibrium) and only report their moments; a link of a
// fluid cell whose source is a solid takes the cell's own post-collision
// population of the opposite link (halfway bounce-back, lbm.cpp:267-274,
// wall at rest).
template <class T, bool FORCED, bool SOLID>
__global__ void __launch_bounds__(256) k_step2d(const T *__restrict__ A, T *__restrict__ B,
                                                const __grid_constant__ Params2 P, State2 *__restrict__ ds,
                                                float *__restrict__ mom, float *__restrict__ band, int gather,
                                                int export_only, int drift, int region, int4 nbx) {
    // launched behind the previous step's IBM pass (programmatic dependent
    // launch): wait for its results first
    cudaGridDependencySynchronize();
    // region 0: every cell; 1: all but the near box nbx (x0, y0, w, h: the IBM
    // box and one cell around it); 2: the near box only, over a grid of its size
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (region == 2) {
        if (x >= nbx.z || y >= nbx.w) return;
        x += nbx.x;
        y += nbx.y;
    }
    if (x >= P.nx || y >= P.ny) return;
    if (region == 1 && (unsigned)(x - nbx.x) < (unsigned)nbx.z && (unsigned)(y - nbx.y) < (unsigned)nbx.w) return;
    const long long cell = x + (long long)P.nx * y;
    float f[Q9];
    const bool face = x == 0 || x == P.nx - 1 || y == 0 || y == P.ny - 1;
    const uint32_t lk = SOLID ? (uint32_t)P.links[cell] : 0u;
    if (SOLID && (lk & kSolidCell)) {
        if (mom != nullptr) {
            float drho = 0.0f, jx = 0.0f, jy = 0.0f;
#pragma unroll
            for (int l = 0; l < Q9; l++) {
                const float v = St<T>::ld(A + l * P.S + cell);
                drho += v;
                jx += (float)cx9(l) * v;
                jy += (float)cy9(l) * v;
            }
            const float rho = 1.0f + drho;
            mom[cell] = rho;
            mom[P.N + cell] = jx / rho;
            mom[2 * P.N + cell] = jy / rho;
        }
        return;
    }
    if (SOLID && gather && (lk & kSolidLinks)) {
        int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0);
        raw &= ~(((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0));
        const Class2 &ce = drift ? P.cls_w[raw] : P.cls[raw];
#pragma unroll
        for (int l = 0; l < Q9; l++)
            f[l] = ((lk >> l) & 1u) ? St<T>::ld(A + opp9(l) * P.S + cell) : pull_link2<T>(A, l, x, y, cell, ce, P);
    } else if (!gather) {
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(A + l * P.S + cell);
    } else if (!face) {
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(A + l * P.S + cell + P.pofs[l]);
    } else {
        int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0);
        raw &= ~(((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0));
        const Class2 &ce = drift ? P.cls_w[raw] : P.cls[raw];
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = pull_link2<T>(A, l, x, y, cell, ce, P);
    }
    float drho = 0.0f, jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        drho += f[l];
        jx += (float)cx9(l) * f[l];
        jy += (float)cy9(l) * f[l];
    }
    const float Fx = FORCED ? P.body[0] : 0.0f, Fy = FORCED ? P.body[1] : 0.0f;
    const float rho = 1.0f + drho;
    const float inv = 1.0f / rho;
    // before the first streaming the stored set-up velocity is used as is
    // (LBM::Init, lbm.cpp:31-57); MacroProp adds F/2 afterwards (lbm.cpp:677-679)
    const float hf = gather ? 0.5f : 0.0f;
    const float ux = (jx + hf * Fx) * inv, uy = (jy + hf * Fy) * inv;
    status_once(&ds->status, lbmk::ST_RHO_RANGE, !(rho > 0.0f && rho < 100.0f));
    if (mom != nullptr) {
        mom[cell] = rho;
        mom[P.N + cell] = ux;
        mom[2 * P.N + cell] = uy;
    }
    if (export_only) return;
    if (P.band_on) {
        const int bx = x - ds->box_lo[0], by = y - ds->box_lo[1];
        if ((unsigned)bx < (unsigned)ds->box_w && (unsigned)by < (unsigned)ds->box_h) {
            // the IBM pass collides this cell: hand over the unforced moments
            // (lbm.cpp:1262-1285) and keep the populations
            const long long b = bx + (long long)P.bsx * by, nb = P.nb;
            band[b] = drho;
            band[nb + b] = ux;
            band[2 * nb + b] = uy;
            band[3 * nb + b] = Fx;
            band[4 * nb + b] = Fy;
#pragma unroll
            for (int l = 0; l < Q9; l++) St<T>::st(B + l * P.S + cell, f[l]);
            return;
        }
    }
    collide9(f, drho, ux, uy, Fx, Fy, P.omega, FORCED);
#pragma unroll
    for (int l = 0; l < Q9; l++) St<T>::st(B + l * P.S + cell, f[l]);
}

// MORE_DETAILS on D2Q9 (LBM.h:55): of the current (streamed) state, the
// pressure p = rho / 3 (lbm.cpp:683) and the viscous stress
// sigma_ab = -(tau - 1/2)/tau sum_l f_l (c_la - u_a)(c_lb - u_b)
// (lbm.cpp:687-705) from the raw second moment,
//     sum f (c - u)(c - u)^T = Pi - u j^T - j u^T + rho u u^T,
// with rho and u of the moment export that precedes it (the shifted storage
// adds c_s^2 to Pi_xx and Pi_yy only: the D2Q9 links have c_z = 0, and u_z
// is zero); with a sample to fold in, Sup_MacroProp's running statistics
// (lbm.cpp:865-939) in FP64, as the D3Q19 pass keeps them.  Layouts
// [component][cell]: details p, sigma xx, xy, xz, yy, yz, zz; statistics
// avg u (3), avg p, avg Reynolds stress (6), rms u (3), rms p, rms Reynolds
// stress (6).
template <class T, bool SOLID>
__global__ void __launch_bounds__(256) k_details2d(const T *__restrict__ A, const __grid_constant__ Params2 P,
                                                   const float *__restrict__ mom, float *__restrict__ det,
                                                   double *__restrict__ st, float sfac, int gather, int drift,
                                                   int fold, double told, double dt) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.nx || y >= P.ny) return;
    const long long cell = x + (long long)P.nx * y;
    float f[Q9];
    const uint32_t lk = SOLID ? (uint32_t)P.links[cell] : 0u;
    int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0);
    raw &= ~(((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0));
    const Class2 &ce = drift ? P.cls_w[raw] : P.cls[raw];
    if (SOLID && (lk & kSolidCell)) {
        // a solid cell keeps its populations (they are its own moments)
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(A + l * P.S + cell);
    } else if (!gather) {
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(A + l * P.S + cell);
    } else {
#pragma unroll
        for (int l = 0; l < Q9; l++)
            f[l] = (SOLID && ((lk >> l) & 1u)) ? St<T>::ld(A + opp9(l) * P.S + cell)
                                              : pull_link2<T>(A, l, x, y, cell, ce, P);
    }
    float jx = 0.0f, jy = 0.0f, pxx = 0.0f, pxy = 0.0f, pyy = 0.0f;
#pragma unroll
    for (int l = 1; l < Q9; l++) {
        const float v = f[l], ex = (float)cx9(l), ey = (float)cy9(l);
        jx += ex * v;
        jy += ey * v;
        pxx += ex * ex * v;
        pxy += ex * ey * v;
        pyy += ey * ey * v;
    }
    const long long N = P.N;
    const float rho = mom[cell], ux = mom[N + cell], uy = mom[2 * N + cell];
    const float cs2 = 1.0f / 3.0f;
    const float sxx = (pxx + cs2) - 2.0f * ux * jx + rho * ux * ux;
    const float syy = (pyy + cs2) - 2.0f * uy * jy + rho * uy * uy;
    const float sxy = pxy - ux * jy - jx * uy + rho * ux * uy;
    det[cell] = rho / 3.0f;
    det[N + cell] = sfac * sxx;
    det[2 * N + cell] = sfac * sxy;
    det[3 * N + cell] = 0.0f;
    det[4 * N + cell] = sfac * syy;
    det[5 * N + cell] = 0.0f;
    det[6 * N + cell] = 0.0f;
    if (!fold) return;
    // Sup_MacroProp, in the reference's order and with its weights
    const double w1 = told + 1.0;
    const double u[3] = {ux, uy, 0.0};
    const double p = (double)rho / 3.0;
    double au[3], d[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        au[a] = (st[a * N + cell] * told + u[a] * dt) / (told + dt);
        st[a * N + cell] = au[a];
        d[a] = u[a] - au[a];
    }
    const double ap = (st[3 * N + cell] * told + p) / w1;
    st[3 * N + cell] = ap;
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    double ars[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
        ars[s] = (st[(4 + s) * N + cell] * told + d[ia[s]] * d[ib[s]]) / w1;
        st[(4 + s) * N + cell] = ars[s];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double r = st[(10 + a) * N + cell];
        st[(10 + a) * N + cell] = sqrt((r * r * told + d[a] * d[a]) / w1);
    }
    // the pressure rms squares the current pressure (lbm.cpp:913)
    const double dp = p - ap;
    st[13 * N + cell] = sqrt((p * p * told + dp * dp) / w1);
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const double r = st[(14 + s) * N + cell];
        const double e = u[ia[s]] * u[ib[s]] - ars[s];
        st[(14 + s) * N + cell] = sqrt((r * r * told + e * e) / w1);
    }
}

// Momentum exchange over a box of the current state (MEA_CL / MEA_CD,
// lbm.cpp:3085-3163): over the fluid cells of the box, every link l whose
// source x - c_l is a solid adds (f*_l + f_opp(l)) c_l, with f* the cell's
// post-collision populations of the last step (the buffer the next step
// pulls from) and f_opp(l) that step's streamed population, pulled here from
// the same buffer (its source x + c_l bounces back f*_l when it is a solid).
// Shifted storage adds 2 w_l.  One block: each thread sums its cells in
// order, then a fixed tree, so the result does not depend on scheduling.
// out = -sum (the force on the body).
template <class T>
__global__ void __launch_bounds__(256) k_mea2d(const T *__restrict__ A, const __grid_constant__ Params2 P, int x0,
                                               int x1, int y0, int y1, double *__restrict__ out, int drift) {
    __shared__ double sp[2][256];
    double px = 0.0, py = 0.0;
    const int bw = x1 - x0 + 1, bh = y1 - y0 + 1;
    const long long n = (bw > 0 && bh > 0) ? (long long)bw * bh : 0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = x0 + (int)(i % bw), y = y0 + (int)(i / bw);
        const long long cell = x + (long long)P.nx * y;
        const uint32_t lk = P.links[cell];
        if ((lk & kSolidCell) || !(lk & kSolidLinks)) continue;
        int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0);
        raw &= ~(((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0));
        const Class2 &ce = drift ? P.cls_w[raw] : P.cls[raw];
        float cpx = 0.0f, cpy = 0.0f;
#pragma unroll
        for (int l = 1; l < Q9; l++) {
            if (!((lk >> l) & 1u)) continue;
            const int o = opp9(l);
            const float fo = ((lk >> o) & 1u) ? St<T>::ld(A + l * P.S + cell) : pull_link2<T>(A, o, x, y, cell, ce, P);
            const float t = St<T>::ld(A + l * P.S + cell) + fo + 2.0f * w9f(l);
            cpx += t * (float)cx9(l);
            cpy += t * (float)cy9(l);
        }
        px += (double)cpx;
        py += (double)cpy;
    }
    sp[0][threadIdx.x] = px;
    sp[1][threadIdx.x] = py;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            sp[0][threadIdx.x] += sp[0][threadIdx.x + h];
            sp[1][threadIdx.x] += sp[1][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = -sp[0][0];
        out[1] = -sp[1][0];
        out[2] = 0.0;
    }
}

// f = feq(rho, u) (LBM::Init, lbm.cpp:31-57), shifted; fields [3][N] or null
// (uniform init[3]).
template <class T>
__global__ void k_init2d(T *__restrict__ A, long long N, long long S, const float *__restrict__ fields,
                         float rho0, float ux0, float uy0) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const float rho = fields ? fields[c] : rho0;
    const float ux = fields ? fields[N + c] : ux0, uy = fields ? fields[2 * N + c] : uy0;
    const float usq = ux * ux + uy * uy;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        const float cu = (float)cx9(l) * ux + (float)cy9(l) * uy;
        const float poly = 3.0f * cu + 4.5f * cu * cu - 1.5f * usq + 4.5f * cu * cu * cu - 4.5f * cu * usq;
        St<T>::st(A + l * S + c, w9f(l) * ((rho - 1.0f) + rho * poly));
    }
}

// ---------------------------------------------------------------------------
// ENERGY: temperature populations on the flow lattice (LBM.h:58)
// ---------------------------------------------------------------------------
// The cubic equilibrium polynomial of Calc_feq / Calc_geq (lbm.cpp:636-653)
// minus one, cs^2 = 1/3.
__device__ __forceinline__ float poly9(float cu, float usq) {
    return 3.0f * cu + 4.5f * cu * cu - 1.5f * usq + 4.5f * cu * cu * cu - 4.5f * cu * usq;
}

// One fused step of f and g.  Streaming (lbm.cpp:263-280): g follows f
// into fluid cells; a link from a Dirichlet wall takes
// -g*_opp(l) + 2 geq_opp(l)(rho, T_w, u_w) of the cell itself, rho of the
// previous MacroProp.  MacroProp (lbm.cpp:668-792): rho, u, T = sum g and
// q = sum g c.  ConvLBM (lbm.cpp:91-177): f by BGK + Guo; g by BGK with the
// viscous-heating source F_l = w_l Phi / cp (1 + c_l.u (tau_g - 1/2) /
// (cs2 tau_g)) plus half its change since the previous collision, where
// Phi = 2 nu rho S:S and S = -sum c c (f - feq) / (2 rho tau cs2).
// aux[N] (one float4 per cell, read once at the top and written once at the
// end) keeps what the previous collision used: rho - 1, u and Phi (the
// reference's F_vis history, F_vis = 0 before the first one).
// ENERGY handles keep f and g in FP32: with geq = rho w T (lbm.cpp:646-650)
// and T = sum g, each collision scales T by 1 + (rho - 1) / tau_g, so T
// integrates any error of rho -- with FP16 f the Couette run's T drifted by
// several times its viscous-heating signal in 2000 steps.
template <class T, bool FORCED>
__global__ void __launch_bounds__(256) k_energy2d(const T *__restrict__ A, T *__restrict__ B,
                                                  const float *__restrict__ GA, float *__restrict__ GB,
                                                  const __grid_constant__ Params2 P,
                                                  const __grid_constant__ Energy2 E, State2 *__restrict__ ds,
                                                  float4 *__restrict__ aux, float *__restrict__ mom, int gather,
                                                  int first, int export_only, int drift) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= P.nx || y >= P.ny) return;
    const long long cell = x + (long long)P.nx * y;
    float f[Q9], g[Q9];
    const bool face = x == 0 || x == P.nx - 1 || y == 0 || y == P.ny - 1;
    const float4 hist = aux[cell];
    const float drho_p = hist.x;
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q9; l++) {
            f[l] = St<T>::ld(A + l * P.S + cell);
            g[l] = GA[l * P.S + cell];
        }
        // Neumann and adiabatic walls: the initial values are the first kept ones
        if (E.gold != nullptr && face && !export_only) {
#pragma unroll
            for (int l = 0; l < Q9; l++) E.gold[l * P.S + cell] = g[l];
        }
    } else if (!face) {
#pragma unroll
        for (int l = 0; l < Q9; l++) {
            f[l] = St<T>::ld(A + l * P.S + cell + P.pofs[l]);
            g[l] = GA[l * P.S + cell + P.pofs[l]];
        }
    } else {
        int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0);
        raw &= ~(((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0));
        const Class2 &ce = drift ? P.cls_w[raw] : P.cls[raw];
        const float *pm1 = drift ? E.pm1_w[raw] : E.pm1[raw];
        const int k = first ? 0 : 1;
        const float tw = E.tw[raw][k], dtw = E.dtw[raw][k];
        const uint32_t neu = E.neu[raw], adi = E.adi[raw];
        float sn = 0.0f;  // Neumann: sum over the other links of (g - w T_ref) c.n
#pragma unroll
        for (int l = 0; l < Q9; l++) {
            f[l] = pull_link2<T>(A, l, x, y, cell, ce, P);
            if ((E.dir[raw] >> l) & 1u) {
                // 2 geq - 2 w T_ref = 2 w (rho T_w (1 + pm1) - T_ref)
                const float wall = 2.0f * w9f(l) * (dtw + drho_p * tw + (1.0f + drho_p) * tw * pm1[l]);
                g[l] = wall - GA[opp9(l) * P.S + cell];
            } else if ((adi >> l) & 1u) {
                g[l] = E.gold[l * P.S + cell];  // never streamed: the initial value
            } else if ((neu >> l) & 1u) {
                g[l] = 0.0f;  // set from T_w below
            } else {
                // a periodic or interior source (the only other links of an
                // ENERGY handle)
                g[l] = pull_link2<float>(GA, l, x, y, cell, ce, P);
                if (neu) {
                    // The reference pushes cell by cell, i outer and j inner,
                    // and forms T_w in the middle of this cell's push: a link
                    // whose source it visited earlier (periodic wrap included;
                    // the rest link in this cell's own push) holds this
                    // sweep's value, the others the previous sweep's.
                    int sx = x - cx9(l), sy = y - cy9(l);
                    sx += sx < 0 ? P.nx : (sx >= P.nx ? -P.nx : 0);
                    sy += sy < 0 ? P.ny : (sy >= P.ny ? -P.ny : 0);
                    const bool fresh = l == 0 || sx < x || (sx == x && sy < y);
                    float *kept = E.gold + l * P.S + cell;
                    sn += (fresh ? g[l] : *kept) * E.cn[raw][l];
                    if (!export_only) *kept = g[l];
                }
            }
        }
        if (neu) {
            // T_w = (j.n - sum_other g c.n) / sum_wall geq(rho, T = 1, u_w) c.n
            // with j.n = 0 (LBM.h's j_dot_n), rho of the previous MacroProp;
            // the wall links take the second-order equilibrium of T_w
            // (lbm.cpp:281-288)
            const float rho_p = 1.0f + drho_p;
            const float Tw = -(sn + E.T_ref * E.nk[raw]) / (rho_p * E.nd[raw]);
#pragma unroll
            for (int l = 0; l < Q9; l++)
                if ((neu >> l) & 1u) g[l] = w9f(l) * (rho_p * Tw * E.nq[raw][l] - E.T_ref);
        }
    }
    float drho = 0.0f, jx = 0.0f, jy = 0.0f, dT = 0.0f, qx = 0.0f, qy = 0.0f;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        drho += f[l];
        jx += (float)cx9(l) * f[l];
        jy += (float)cy9(l) * f[l];
        dT += g[l];
        qx += (float)cx9(l) * g[l];
        qy += (float)cy9(l) * g[l];
    }
    // before the first MacroProp the collision takes the set-up T (uniform,
    // the shift T_ref)
    if (!gather) dT = 0.0f;
    const float Fx = FORCED ? P.body[0] : 0.0f, Fy = FORCED ? P.body[1] : 0.0f;
    const float rho = 1.0f + drho;
    const float inv = 1.0f / rho;
    const float hf = gather ? 0.5f : 0.0f;
    const float ux = (jx + hf * Fx) * inv, uy = (jy + hf * Fy) * inv;
    const float Tc = E.T_ref + dT;
    status_once(&ds->status, lbmk::ST_RHO_RANGE, !(rho > 0.0f && rho < 100.0f));
    status_once(&ds->status, lbmk::ST_T_RANGE, !(Tc > 0.0f && Tc < 100.0f));
    if (mom != nullptr) {
        mom[cell] = rho;
        mom[P.N + cell] = ux;
        mom[2 * P.N + cell] = uy;
        mom[3 * P.N + cell] = Tc;
        mom[4 * P.N + cell] = qx;  // sum g c: the shift w T_ref carries no momentum
        mom[5 * P.N + cell] = qy;
    }
    if (export_only) return;
    const float usq = ux * ux + uy * uy;
    float sxx = 0.0f, sxy = 0.0f, syy = 0.0f;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        const float cu = (float)cx9(l) * ux + (float)cy9(l) * uy;
        const float fne = f[l] - w9f(l) * (drho + rho * poly9(cu, usq));
        sxx += (float)(cx9(l) * cx9(l)) * fne;
        sxy += (float)(cx9(l) * cy9(l)) * fne;
        syy += (float)(cy9(l) * cy9(l)) * fne;
    }
    const float sk = E.s_fac * inv;
    sxx *= sk;
    sxy *= sk;
    syy *= sk;
    const float phi = E.two_nu * rho * (sxx * sxx + 2.0f * sxy * sxy + syy * syy);
    const float uxp = hist.y, uyp = hist.z, phip = hist.w;
    collide9(f, drho, ux, uy, Fx, Fy, P.omega, FORCED);
    const float a = phi * E.inv_cp, ap = phip * E.inv_cp;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        const float cu = (float)cx9(l) * ux + (float)cy9(l) * uy;
        const float cup = (float)cx9(l) * uxp + (float)cy9(l) * uyp;
        const float Fl = w9f(l) * a * (1.0f + cu * E.tg_fac);
        const float Fb = w9f(l) * ap * (1.0f + cup * E.tg_fac);
        const float geq_s = w9f(l) * (dT + drho * Tc + rho * Tc * poly9(cu, usq));
        g[l] = g[l] - (g[l] - geq_s) * E.inv_tau_g + Fl + 0.5f * (Fl - Fb);
    }
    aux[cell] = make_float4(drho, ux, uy, phi);
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        St<T>::st(B + l * P.S + cell, f[l]);
        GB[l * P.S + cell] = g[l];
    }
}

// g = geq(rho, u, T0) (LBM::Init, lbm.cpp:44-49), shifted by w T0 with T0
// the uniform set-up T; aux = (rho - 1, u, Phi = 0).
__global__ void k_init_energy2d(float *__restrict__ G, float4 *__restrict__ aux, long long N, long long S,
                                const float *__restrict__ fields, float rho0, float ux0, float uy0, float T0) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const float rho = fields ? fields[c] : rho0;
    const float ux = fields ? fields[N + c] : ux0, uy = fields ? fields[2 * N + c] : uy0;
    const float usq = ux * ux + uy * uy;
#pragma unroll
    for (int l = 0; l < Q9; l++) {
        const float cu = (float)cx9(l) * ux + (float)cy9(l) * uy;
        G[l * S + c] = w9f(l) * ((rho - 1.0f) * T0 + rho * T0 * poly9(cu, usq));
    }
    aux[c] = make_float4(rho - 1.0f, ux, uy, 0.0f);
}

// ---------------------------------------------------------------------------
// Immersed boundary
// ---------------------------------------------------------------------------
struct Ibm2 {
    int n, m_max, lit_sign, rho_nearest, added_mass, motion, scheme;
    double Dbox;     // the box reaches centre -/+ Dbox (the body diameter, lbm.cpp:1165-1166)
    double vsolid, amp, freq;
    double vconst[3];
    double *pos;      // [3][n] reference node coordinates
    const double *nrm;  // [3][n]
    const double *dsw;  // [n]
    float *fs;        // [2][n] F_m ds_m of the current iteration
    float *rhom;      // [n]
    int *s0;          // [2][n] stencil origin, box coordinates
    float *swt;       // [16][n] stencil weights (0 outside the box)
    int *cnt, *off;   // [nb], [nb]
    int *lm;          // [16 n] spreading lists: marker
    float *lw;        //                         weight
    int *qnear;       // [n] nearest box node of each marker (band index), -1 for none
    uint8_t *inside;  // [nb] box node inside every marker (Calc_AverageDensity)
    float *boxF;      // [4][nb] force and forced velocity the box cells collided with (fluid[..].F,
                      // ux, uy after IBLBM), box order
    double *hist;     // [cap][4]: drag, lift, 0, step
    int smem;         // 1: the working fields of the pass live in shared memory
    int fast;         // 1: box nodes in registers (at most kFastNodes per thread, n <= block size)
};

// Box nodes a thread of the register-resident pass owns.
constexpr int kFastNodes = 4;

// Shared-memory words of the register-resident pass: u at the box nodes
// (2 nb), the marker forces (2 n), the stencils as (node, weight) pairs
// (32 n), the spreading lists as (marker, weight) pairs (32 n), the marker
// densities (n), the box nodes with a spreading list (nb).
__host__ __device__ inline size_t ibm2d_fast_smem_bytes(long long nb, int n) {
    return (size_t)4 * (3 * (size_t)nb + 67 * (size_t)n);
}

// 4-point Peskin delta (lbm.cpp:1095-1102).
__device__ __forceinline__ double peskin_d(double r) {
    const double a = fabs(r);
    if (a <= 1.0) return (3.0 - 2.0 * a + sqrt(1.0 + 4.0 * a - 4.0 * r * r)) / 8.0;
    if (a <= 2.0) return (5.0 - 2.0 * a - sqrt(-7.0 + 12.0 * a - 4.0 * r * r)) / 8.0;
    return 0.0;
}

// V_CM(t) of the prescribed motions (lbm.cpp:1140-1151).
__device__ __forceinline__ void motion_velocity(const Ibm2 &ib, double t, double V[3]) {
    V[0] = V[1] = V[2] = 0.0;
    if (ib.motion == LBM_MOTION_CONSTANT) {
        V[0] = ib.vconst[0];
        V[1] = ib.vconst[1];
        V[2] = ib.vconst[2];
    } else if (ib.motion == LBM_MOTION_INLINE_OSC) {
        V[0] = -ib.amp * cos(2.0 * kRefPi * ib.freq * t);
    } else if (ib.motion == LBM_MOTION_TRANSVERSE_OSC) {
        V[1] = -2.0 * kRefPi * ib.freq * ib.amp * sin(2.0 * kRefPi * ib.freq * t);
    }
}

// The kinematics of IBLBM for reference step s (lbm.cpp:1137-1167): V_CM
// of step s and of the step before, the centre moved by the trapezoid, and
// the box [floor(c - D), ceil(c + D)] (z = 1).  box_of only computes the box
// of step s (for the collide-stream launch that precedes the IBM pass);
// advance_body commits the step (V, centre, markers, desired velocity) at
// the start of the pass.  Both evaluate V(s) and the centre with the same
// operations, so the box matches the committed centre.
__device__ void box_of(State2 *st, const Ibm2 &ib, const Params2 &P, long long s) {
    double V[3], c[2];
    motion_velocity(ib, (double)s, V);
    for (int a = 0; a < 2; a++) c[a] = st->center[a] + (V[a] + st->V[a]) * 1.0 / 2;
    const int xmin = (int)floor(c[0] - ib.Dbox), xmax = (int)ceil(c[0] + ib.Dbox);
    const int ymin = (int)floor(c[1] - ib.Dbox), ymax = (int)ceil(c[1] + ib.Dbox);
    // reference node i is device cell i - 1; the box must lie in the interior
    int lo0 = xmin - 1, lo1 = ymin - 1, w = xmax - xmin + 1, hgt = ymax - ymin + 1;
    if (lo0 < 0 || lo1 < 0 || lo0 + w > P.nx || lo1 + hgt > P.ny || w > P.bsx || hgt > P.bsy) {
        atomicOr(&st->status, lbmk::ST_BAND_EDGE);
        lo0 = max(lo0, 0);
        lo1 = max(lo1, 0);
        w = min(min(w, P.bsx), P.nx - lo0);
        hgt = min(min(hgt, P.bsy), P.ny - lo1);
    }
    st->box_lo[0] = lo0;
    st->box_lo[1] = lo1;
    st->box_w = w;
    st->box_h = hgt;
}

// One thread: V_CM of step s and the centre (the markers were moved by
// k_move2d).
__device__ void advance_body(State2 *st, const Ibm2 &ib, long long s) {
    double V[3];
    motion_velocity(ib, (double)s, V);
    for (int a = 0; a < 3; a++) {
        const double vo = st->V[a];
        st->Vold[a] = vo;
        st->V[a] = V[a];
        st->center[a] += (V[a] + vo) * 1.0 / 2;
    }
    st->ibm_step = s;
    if (ib.motion != LBM_MOTION_FIXED) st->lists_ok = 0;
}

// The box of reference step 1, before its collide-stream launch.
__global__ void k_kin2d(State2 *st, Ibm2 ib, const __grid_constant__ Params2 P) { box_of(st, ib, P, 1); }

// Block-wide exclusive scan of one int per thread (blockDim 1024).
__device__ int block_scan(int v, int *total) {
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    const int before = (w > 0 ? wsum[w - 1] : 0) + x - v;
    *total = wsum[31];
    __syncthreads();
    return before;
}

// Two FP64 block sums in a fixed order (warp shuffles, then thread 0 over the
// warps' partials, the two sums as independent chains).
__device__ void block_sum_d2(double a, double b, double &sa, double &sb) {
    __shared__ double part[2][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
        part[0][w] = a;
        part[1][w] = b;
    }
    __syncthreads();
    double x = 0.0, y = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
            x += part[0][i];
            y += part[1][i];
        }
    __syncthreads();
    sa = x;  // valid in thread 0
    sb = y;
}

// Marker m's stencil: origin (box coordinates) and the 16 weights
// kernel(rx) kernel(ry) kernel(rz) of the box nodes i = floor(X)-1 .. +2
// (x outer), j likewise, k = 1 (lbm.cpp:1288-1309); 0 outside the box.
__device__ __forceinline__ void marker_stencil(const Ibm2 &ib, const State2 *st, int m) {
    const int n = ib.n;
    const double X = ib.pos[m], Y = ib.pos[n + m], Z = ib.pos[2 * n + m];
    const int i0 = (int)floor(X) - 1, j0 = (int)floor(Y) - 1;
    // box node (bx, by) is reference node (box_lo + 1 + bx, ...)
    const int bx0 = i0 - (st->box_lo[0] + 1), by0 = j0 - (st->box_lo[1] + 1);
    ib.s0[m] = bx0;
    ib.s0[n + m] = by0;
    const double kz = peskin_d(1.0 - Z);
    for (int a = 0; a < 4; a++) {
        const double kx = peskin_d((double)(i0 + a) - X);
        for (int b = 0; b < 4; b++) {
            const double ky = peskin_d((double)(j0 + b) - Y);
            const bool in = (unsigned)(bx0 + a) < (unsigned)st->box_w && (unsigned)(by0 + b) < (unsigned)st->box_h;
            ib.swt[(4 * a + b) * n + m] = in ? (float)(kx * ky * kz) : 0.0f;
        }
    }
}

// NearestLatticeCoordinate (lbm.cpp:1074-1092) over box nodes
// [xa, xb] x [ya, yb] (box coordinates), one warp: the last node in
// x-outer / y-inner order with the largest (x - X) . n > 0.  Returns the box
// node, or -1 when none lies on the outer side.
__device__ __forceinline__ long long nearest_node(const Ibm2 &ib, const State2 *st, const Params2 &P, int m,
                                                  int xa, int xb, int ya, int yb) {
    const int n = ib.n, lane = threadIdx.x & 31;
    const double X = ib.pos[m], Y = ib.pos[n + m], Z = ib.pos[2 * n + m];
    const double nx = ib.nrm[m], ny = ib.nrm[n + m], nz = ib.nrm[2 * n + m];
    const int w = xb - xa + 1, h = yb - ya + 1;
    double best = 0.0;
    int bo = -1;
    for (int o = lane; o < w * h; o += 32) {
        const int bx = xa + o / h, by = ya + o % h;
        const double d = ((double)(st->box_lo[0] + 1 + bx) - X) * nx + ((double)(st->box_lo[1] + 1 + by) - Y) * ny +
                         (1.0 - Z) * nz;
        if (d >= best && d > 0.0) {
            best = d;
            bo = o;
        }
    }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, s);
        const int oo = __shfl_xor_sync(0xffffffffu, bo, s);
        if (oo >= 0 && (bo < 0 || ob > best || (ob == best && oo > bo))) {
            best = ob;
            bo = oo;
        }
    }
    if (bo < 0) return -1;
    return (long long)(xa + bo / h) + (long long)P.bsx * (ya + bo % h);
}

// Markers of step s (one warp each, many blocks): moved by the trapezoid of
// V_CM (lbm.cpp:1153-1160), and their nearest box node (the whole box, or
// the 2x2 cell around the marker in the explicit scheme, lbm.cpp:1216-1219).
// Runs before the step's collide-stream launch; the box of step s is set.
constexpr int kMoveBlock = 256;
__global__ void __launch_bounds__(kMoveBlock) k_move2d(State2 *__restrict__ st, Ibm2 ib,
                                                       const __grid_constant__ Params2 P) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31, n = ib.n;
    if (m >= n) return;  // whole warp leaves together
    if (ib.motion != LBM_MOTION_FIXED) {
        double V[3];
        motion_velocity(ib, (double)(st->ibm_step + 1), V);
        if (lane == 0)
            for (int a = 0; a < 3; a++) ib.pos[a * n + m] += (V[a] + st->V[a]) * 1.0 / 2;
        __syncwarp();
    }
    if (!ib.rho_nearest) return;
    const int bw = st->box_w, bh = st->box_h;
    int xa = 0, xb = bw - 1, ya = 0, yb = bh - 1;
    if (ib.scheme == 1) {
        const double X = ib.pos[m], Y = ib.pos[n + m];
        xa = (int)floor(X) - (st->box_lo[0] + 1);
        xb = (int)ceil(X) - (st->box_lo[0] + 1);
        ya = (int)floor(Y) - (st->box_lo[1] + 1);
        yb = (int)ceil(Y) - (st->box_lo[1] + 1);
        if (xa < 0 || ya < 0 || xb >= bw || yb >= bh) {
            if (lane == 0) atomicOr(&st->status, lbmk::ST_BAND_EDGE);
            xa = max(xa, 0);
            ya = max(ya, 0);
            xb = min(xb, bw - 1);
            yb = min(yb, bh - 1);
        }
    }
    const long long q = nearest_node(ib, st, P, m, xa, xb, ya, yb);
    if (lane == 0) {
        if (q < 0) atomicOr(&st->status, lbmk::ST_BAND_EDGE);
        ib.qnear[m] = (int)q;
    }
}

// Box nodes inside every marker, (x - X_m) . n_m <= 0 for all m
// (Calc_AverageDensity, lbm.cpp:1105-1132), for the added mass of a moving
// body; after k_move2d.
__global__ void __launch_bounds__(kMoveBlock) k_inside2d(const State2 *__restrict__ st, Ibm2 ib,
                                                         const __grid_constant__ Params2 P) {
    const int bw = st->box_w, bh = st->box_h, n = ib.n;
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= bw * bh) return;
    const int bx = o % bw, by = o / bw;
    const double X = (double)(st->box_lo[0] + 1 + bx), Y = (double)(st->box_lo[1] + 1 + by);
    bool inside = true;
    for (int m = 0; m < n && inside; m++) {
        const double d = (X - ib.pos[m]) * ib.nrm[m] + (Y - ib.pos[n + m]) * ib.nrm[n + m] +
                         (1.0 - ib.pos[2 * n + m]) * ib.nrm[2 * n + m];
        if (d > 0.0) inside = false;
    }
    ib.inside[bx + (long long)P.bsx * by] = inside ? 1 : 0;
}

// Shared-memory bytes of the working fields of one pass: the box fields
// (rho, u, F: 5 nb floats), list offsets and counts (2 nb), lists (2 x 16 n),
// marker forces, densities, stencil origins and weights (21 n).
__host__ __device__ inline size_t ibm2d_smem_bytes(long long nb, int n) {
    return (size_t)4 * (7 * (size_t)nb + 53 * (size_t)n);
}

template <class T>
__global__ void __launch_bounds__(kIbmBlock) k_ibm2d(T *__restrict__ B, const __grid_constant__ Params2 P,
                                                     State2 *__restrict__ st, Ibm2 ib, float *__restrict__ band) {
    extern __shared__ float smem[];
    // launched behind the collide-stream grid (programmatic dependent launch)
    cudaGridDependencySynchronize();
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n = ib.n;
    const long long nb = P.nb;
    // IBLBM's prelude for this step: V_CM and the centre (the markers were
    // moved and the box set before the collide-stream launch)
    const long long step = st->ibm_step + 1;
    __syncthreads();
    if (tid == 0) advance_body(st, ib, step);
    __syncthreads();
    const int bw = st->box_w, bh = st->box_h, nbox = bw * bh;
    // the box this pass collides, for the force-density output (boxF)
    if (tid == 0) {
        st->fbox[0] = st->box_lo[0];
        st->fbox[1] = st->box_lo[1];
        st->fbox[2] = bw;
        st->fbox[3] = bh;
    }
    const int lists_ok = st->lists_ok;
    const float V0 = (float)st->V[0], V1 = (float)st->V[1];
    auto bq = [&](int o) { return (long long)(o % bw) + (long long)P.bsx * (o / bw); };
    __syncthreads();

    // stencils and spreading lists, in global scratch (fixed body: once)
    if (!lists_ok) {
        for (int m = tid; m < n; m += nt) marker_stencil(ib, st, m);
        for (int o = tid; o < nbox; o += nt) ib.cnt[bq(o)] = 0;
        __syncthreads();
        for (int m = tid; m < n; m += nt)
            for (int k = 0; k < 16; k++)
                if (ib.swt[k * n + m] != 0.0f)
                    atomicAdd(&ib.cnt[(ib.s0[m] + k / 4) + (long long)P.bsx * (ib.s0[n + m] + k % 4)], 1);
        __syncthreads();
        // offsets: contiguous chunks of box nodes per thread, then a block scan
        const int chunk = (nbox + nt - 1) / nt, o0 = tid * chunk, o1 = min(nbox, o0 + chunk);
        int mine = 0;
        for (int o = o0; o < o1; o++) mine += ib.cnt[bq(o)];
        int total;
        int run = block_scan(mine, &total);
        for (int o = o0; o < o1; o++) {
            const long long q = bq(o);
            ib.off[q] = run;
            run += ib.cnt[q];
            ib.cnt[q] = 0;
        }
        __syncthreads();
        for (int m = tid; m < n; m += nt)
            for (int k = 0; k < 16; k++) {
                const float w = ib.swt[k * n + m];
                if (w == 0.0f) continue;
                const long long q = (ib.s0[m] + k / 4) + (long long)P.bsx * (ib.s0[n + m] + k % 4);
                const int slot = ib.off[q] + atomicAdd(&ib.cnt[q], 1);
                ib.lm[slot] = m;
                ib.lw[slot] = w;
            }
        __syncthreads();
        // ascending marker order in every list (the reference's summation order)
        for (int o = tid; o < nbox; o += nt) {
            const long long q = bq(o);
            const int a = ib.off[q], c = ib.cnt[q];
            for (int i = 1; i < c; i++) {
                const int km = ib.lm[a + i];
                const float kw = ib.lw[a + i];
                int j = i - 1;
                while (j >= 0 && ib.lm[a + j] > km) {
                    ib.lm[a + j + 1] = ib.lm[a + j];
                    ib.lw[a + j + 1] = ib.lw[a + j];
                    j--;
                }
                ib.lm[a + j + 1] = km;
                ib.lw[a + j + 1] = kw;
            }
        }
        if (tid == 0 && ib.motion == LBM_MOTION_FIXED) st->lists_ok = 1;
        __syncthreads();
    }

    const float sgn = ib.lit_sign ? -1.0f : 1.0f;
    double drag, lift;
    if (ib.fast) {
        // Register-resident pass over the box nodes some marker spreads to
        // (the others keep their u and F through the iterations): every
        // thread keeps its nodes' index, 1 / (2 rho), u, F and list span in
        // registers for the m_max iterations; shared memory holds u (read by
        // the interpolation, which reads only these nodes), the marker
        // forces, the stencils and the lists as packed pairs.
        float2 *uxy = reinterpret_cast<float2 *>(smem);
        float2 *fsp = uxy + nb;
        float2 *mst = fsp + n;                               // [16][n] (node as int bits, weight)
        int2 *lst = reinterpret_cast<int2 *>(mst + 16 * n);  // (marker, weight as int bits)
        float *rhm = reinterpret_cast<float *>(lst + 16 * n);
        int *act = reinterpret_cast<int *>(rhm + n);         // box order of the nodes with a list
        int nact;
        {
            const int chunk = (nbox + nt - 1) / nt, o0 = tid * chunk, o1 = min(nbox, o0 + chunk);
            int mine = 0;
            for (int o = o0; o < o1; o++) mine += ib.cnt[bq(o)] > 0 ? 1 : 0;
            int run = block_scan(mine, &nact);
            for (int o = o0; o < o1; o++)
                if (ib.cnt[bq(o)] > 0) act[run++] = o;
        }
        __syncthreads();
        int nq[kFastNodes], la[kFastNodes], lc[kFastNodes];
        float hr[kFastNodes], fx[kFastNodes], fy[kFastNodes], vx[kFastNodes], vy[kFastNodes];
#pragma unroll
        for (int k = 0; k < kFastNodes; k++) {
            const int a = tid + k * nt;
            nq[k] = -1;
            la[k] = lc[k] = 0;
            hr[k] = fx[k] = fy[k] = vx[k] = vy[k] = 0.0f;
            if (a < nact) {
                const int q = (int)bq(act[a]);
                nq[k] = q;
                hr[k] = 0.5f / (1.0f + band[q]);
                vx[k] = band[nb + q];
                vy[k] = band[2 * nb + q];
                fx[k] = band[3 * nb + q];
                fy[k] = band[4 * nb + q];
                la[k] = ib.off[q];
                lc[k] = ib.cnt[q];
                uxy[q] = make_float2(vx[k], vy[k]);
            }
        }
        for (int i = tid; i < 16 * n; i += nt) {
            const int k = i / n, m = i - k * n;
            const float w = ib.swt[i];
            const int q = w != 0.0f ? (ib.s0[m] + k / 4) + P.bsx * (ib.s0[n + m] + k % 4) : -1;
            mst[i] = make_float2(__int_as_float(q), w);
            lst[i] = make_int2(ib.lm[i], __float_as_int(ib.lw[i]));
        }
        // marker density: nearest node (k_move2d), or delta-interpolated
        float rmine = 0.0f, dsmine = 0.0f;
        double dsd = 0.0;
        if (tid < n) {
            const int m = tid;
            if (ib.rho_nearest) {
                const int q = ib.qnear[m];
                rmine = q < 0 ? 1.0f : 1.0f + band[q];
            } else {
                float sr = 0.0f;
                for (int k = 0; k < 16; k++) {
                    const float w = ib.swt[k * n + m];
                    if (w != 0.0f) sr += (1.0f + band[(ib.s0[m] + k / 4) + P.bsx * (ib.s0[n + m] + k % 4)]) * w;
                }
                rmine = sr;
            }
            rhm[m] = rmine;
            dsd = ib.dsw[m];
            dsmine = (float)dsd;
        }
        __syncthreads();
        double mk_drag = 0.0, mk_lift = 0.0, node_drag = 0.0, node_lift = 0.0;
        const int iters = ib.scheme == 1 ? 1 : ib.m_max;
        for (int it = 0; it < iters; it++) {
            // interpolation and marker force (lbm.cpp:1314-1324), one
            // thread per marker, nodes in the reference's order
            if (tid < n) {
                const int m = tid;
                float ub = 0.0f, vb = 0.0f;
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const float2 e = mst[k * n + m];
                    const int q = __float_as_int(e.x);
                    if (q >= 0) {
                        const float2 u = uxy[q];
                        ub += u.x * e.y;
                        vb += u.y * e.y;
                    }
                }
                const float Fbx = 2.0f * rmine * (V0 - ub), Fby = 2.0f * rmine * (V1 - vb);
                fsp[m] = make_float2(Fbx * dsmine, Fby * dsmine);
                mk_drag += -(double)Fbx * 1.0 * dsd;
                mk_lift += -(double)Fby * 1.0 * dsd;
                if (!isfinite(Fbx) || !isfinite(Fby)) atomicOr(&st->status, lbmk::ST_NONFINITE_FORCE);
            }
            __syncthreads();
            // spreading onto this thread's nodes, ascending marker order
#pragma unroll
            for (int k = 0; k < kFastNodes; k++) {
                if (nq[k] < 0) continue;
                float sx = 0.0f, sy = 0.0f;
                // unrolled: the list entries' loads overlap (the sum keeps
                // its ascending marker order)
#pragma unroll 4
                for (int i = la[k]; i < la[k] + lc[k]; i++) {
                    const int2 e = lst[i];
                    const float2 f = fsp[e.x];
                    const float w = __int_as_float(e.y);
                    sx += f.x * w;
                    sy += f.y * w;
                }
                if (ib.scheme == 0) {
                    fx[k] += sgn * sx;
                    fy[k] += sgn * sy;
                } else {
                    fx[k] += sx;
                    fy[k] += sy;
                    node_drag += -(double)sx;
                    node_lift += -(double)sy;
                }
                vx[k] += sx * hr[k];
                vy[k] += sy * hr[k];
                uxy[nq[k]] = make_float2(vx[k], vy[k]);
            }
            __syncthreads();
        }
        block_sum_d2(ib.scheme == 0 ? mk_drag : node_drag, ib.scheme == 0 ? mk_lift : node_lift, drag, lift);
        // the forced nodes' u and F back into the box fields, then the
        // collision of every box cell
#pragma unroll
        for (int k = 0; k < kFastNodes; k++) {
            if (nq[k] < 0) continue;
            band[nb + nq[k]] = vx[k];
            band[2 * nb + nq[k]] = vy[k];
            band[3 * nb + nq[k]] = fx[k];
            band[4 * nb + nq[k]] = fy[k];
        }
        __syncthreads();
        for (int o = tid; o < nbox; o += nt) {
            const long long q = bq(o);
            const float ux = band[nb + q], uy = band[2 * nb + q], Fx = band[3 * nb + q], Fy = band[4 * nb + q];
            const long long cell = (st->box_lo[0] + o % bw) + (long long)P.nx * (st->box_lo[1] + o / bw);
            float f[Q9];
#pragma unroll
            for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(B + l * P.S + cell);
            collide9(f, band[q], ux, uy, Fx, Fy, P.omega, true);
            ib.boxF[o] = Fx;
            ib.boxF[P.nb + o] = Fy;
            ib.boxF[2 * P.nb + o] = ux;
            ib.boxF[3 * P.nb + o] = uy;
#pragma unroll
            for (int l = 0; l < Q9; l++) St<T>::st(B + l * P.S + cell, f[l]);
        }
    } else {
    // working copies: shared memory when they fit, else the global arrays
    float *drho = band, *ux = band + nb, *uy = band + 2 * nb, *Fx = band + 3 * nb, *Fy = band + 4 * nb;
    int *cnt = ib.cnt, *off = ib.off, *lm = ib.lm, *s0 = ib.s0;
    float *lw = ib.lw, *swt = ib.swt, *fs = ib.fs, *rhom = ib.rhom;
    if (ib.smem) {
        float *p = smem;
        drho = p; ux = p + nb; uy = p + 2 * nb; Fx = p + 3 * nb; Fy = p + 4 * nb;
        p += 5 * nb;
        cnt = (int *)p; off = (int *)p + nb;
        p += 2 * nb;
        lm = (int *)p; lw = p + 16 * n; fs = p + 32 * n; rhom = p + 34 * n; s0 = (int *)p + 35 * n;
        swt = p + 37 * n;
        for (int o = tid; o < nbox; o += nt) {
            const long long q = bq(o);
            drho[q] = band[q];
            ux[q] = band[nb + q];
            uy[q] = band[2 * nb + q];
            Fx[q] = band[3 * nb + q];
            Fy[q] = band[4 * nb + q];
            cnt[q] = ib.cnt[q];
            off[q] = ib.off[q];
        }
        for (int i = tid; i < 16 * n; i += nt) {
            lm[i] = ib.lm[i];
            lw[i] = ib.lw[i];
            swt[i] = ib.swt[i];
        }
        for (int i = tid; i < 2 * n; i += nt) s0[i] = ib.s0[i];
        __syncthreads();
    }
    auto interp = [&](const float *fa, const float *fb, int m, float &sa, float &sb) {
        const int bx0 = s0[m], by0 = s0[n + m];
        float a0 = 0.0f, b0 = 0.0f;
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) {
                const float w = swt[(4 * a + b) * n + m];
                if (w != 0.0f) {
                    const long long q = (bx0 + a) + (long long)P.bsx * (by0 + b);
                    a0 += fa[q] * w;
                    if (fb) b0 += fb[q] * w;
                }
            }
        sa = a0;
        sb = b0;
    };

    // marker density: nearest node (k_move2d), or delta-interpolated
    for (int m = tid; m < n; m += nt) {
        if (ib.rho_nearest) {
            const int q = ib.qnear[m];
            rhom[m] = q < 0 ? 1.0f : 1.0f + drho[q];
        } else {
            float sr, dummy;
            interp(drho, nullptr, m, sr, dummy);
            float wsum = 0.0f;
            for (int k = 0; k < 16; k++) wsum += swt[k * n + m];
            rhom[m] = wsum + sr;  // sum (1 + drho) delta
        }
    }
    __syncthreads();

    double node_drag = 0.0, node_lift = 0.0, mk_drag = 0.0, mk_lift = 0.0;
    const int iters = ib.scheme == 1 ? 1 : ib.m_max;
    for (int it = 0; it < iters; it++) {
        // interpolate the current velocity; marker forces (lbm.cpp:1314-1324)
        for (int m = tid; m < n; m += nt) {
            float ub, vb;
            interp(ux, uy, m, ub, vb);
            const float rho = rhom[m];
            const float Fbx = 2.0f * rho * (V0 - ub), Fby = 2.0f * rho * (V1 - vb);
            const double dsv = ib.dsw[m];
            fs[m] = (float)(Fbx * dsv);
            fs[n + m] = (float)(Fby * dsv);
            // a thread keeps its markers' FP64 sums over the iterations
            mk_drag += -(double)Fbx * 1.0 * dsv;
            mk_lift += -(double)Fby * 1.0 * dsv;
            if (!isfinite(Fbx) || !isfinite(Fby)) atomicOr(&st->status, lbmk::ST_NONFINITE_FORCE);
        }
        __syncthreads();
        // spreading, node-centred, ascending marker order (lbm.cpp:1331-1352)
        for (int o = tid; o < nbox; o += nt) {
            const long long q = bq(o);
            const int a = off[q], c = cnt[q];
            float sx = 0.0f, sy = 0.0f;
            for (int i = 0; i < c; i++) {
                const int m = lm[a + i];
                const float w = lw[a + i];
                sx += fs[m] * w;
                sy += fs[n + m] * w;
            }
            const float rho = 1.0f + drho[q];
            if (ib.scheme == 0) {
                Fx[q] += sgn * sx;
                Fy[q] += sgn * sy;
            } else {
                // explicit: F = sum F_m ds delta, u += F / 2 rho, Drag -= F dx^2
                Fx[q] += sx;
                Fy[q] += sy;
                node_drag += -(double)sx;
                node_lift += -(double)sy;
            }
            ux[q] += sx / (2.0f * rho);
            uy[q] += sy / (2.0f * rho);
        }
        __syncthreads();
    }

    // the pass's force: sum over markers (implicit) or box nodes (explicit)
    block_sum_d2(ib.scheme == 0 ? mk_drag : node_drag, ib.scheme == 0 ? mk_lift : node_lift, drag, lift);

    // collision of the box cells with the forced velocity and the force
    for (int o = tid; o < nbox; o += nt) {
        const long long q = bq(o);
        const long long cell = (st->box_lo[0] + o % bw) + (long long)P.nx * (st->box_lo[1] + o / bw);
        float f[Q9];
#pragma unroll
        for (int l = 0; l < Q9; l++) f[l] = St<T>::ld(B + l * P.S + cell);
        collide9(f, drho[q], ux[q], uy[q], Fx[q], Fy[q], P.omega, true);
        ib.boxF[o] = Fx[q];
        ib.boxF[P.nb + o] = Fy[q];
        ib.boxF[2 * P.nb + o] = ux[q];
        ib.boxF[3 * P.nb + o] = uy[q];
#pragma unroll
        for (int l = 0; l < Q9; l++) St<T>::st(B + l * P.S + cell, f[l]);
    }
    }  // general pass

    // added mass (lbm.cpp:1392-1398): mean density of the box nodes inside
    // every marker (k_inside2d); skipped when V_CM did not change, where it
    // adds rho_avg * 0
    __shared__ double sam[2];
    const double dV0 = st->V[0] - st->Vold[0], dV1 = st->V[1] - st->Vold[1];
    if (ib.added_mass && (dV0 != 0.0 || dV1 != 0.0)) {
        double rs = 0.0, cn = 0.0;
        for (int o = tid; o < nbox; o += nt) {
            const long long q = bq(o);
            if (ib.inside[q]) {
                rs += 1.0 + (double)band[q];
                cn += 1.0;
            }
        }
        double tr, tc;
        block_sum_d2(rs, cn, tr, tc);
        if (tid == 0) {
            const double ravg = tr / tc;
            sam[0] = ravg * ib.vsolid * dV0 / 1.0;
            sam[1] = ravg * ib.vsolid * dV1 / 1.0;
        }
    } else if (tid == 0) {
        sam[0] = sam[1] = 0.0;
    }
    __syncthreads();
    if (tid == 0) {
        double *row = ib.hist + 4 * ((step - 1) % st->hist_cap);
        row[0] = drag + sam[0];
        row[1] = lift + sam[1];
        row[2] = 0.0;
        row[3] = (double)step;
    }

    __syncthreads();
    // the box of the next step, for its collide-stream launch
    if (tid == 0) box_of(st, ib, P, step + 1);
}

}  // namespace l2d

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
using namespace l2d;

struct lbm2d {
    Params2 P;
    State2 *st = nullptr;
    void *f[2] = {nullptr, nullptr};
    int cur = 0;
    float *mom = nullptr;
    float *band = nullptr;
    bool ibm = false, normals = false, kin_ready = false;
    lbm_ibm_config ic;
    Ibm2 ib;
    double *hist = nullptr;
    long long hist_cap = 1 << 16;
    // lbmgpu_get_forces: pinned, device-mapped rows, grown on demand
    double *fstage = nullptr;
    long long fstage_rows = 0;
    // graphs of gsteps steps, one per parity of the buffer they start from
    // (a graph reads and writes fixed buffers)
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gsteps = 16;
    int tx = 128, ty = 2;
    // ENERGY: g ping-pong, per-cell history of the last collision
    bool energy = false;
    Energy2 E;
    float *g[2] = {nullptr, nullptr};
    float4 *aux = nullptr;
    // interior solid cells: the per-cell link masks, a momentum-exchange result
    uint16_t *links = nullptr;
    double *mea_out = nullptr;
    // a fixed IBM body: the next step's cells away from the box ("far") run
    // beside the IBM pass, which with the near box goes on a second stream
    bool overlap = false, overlap_known = false;
    int4 nbox = make_int4(0, 0, 0, 0);  // near box: x0, y0, w, h
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_far = nullptr, ev_near = nullptr, ev_join = nullptr;
    std::vector<void *> allocs;
};

namespace {

lbm_status f2(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

#define CK2(expr)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) return f2(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

template <class Tp>
cudaError_t alloc2(lbm_handle *h, Tp **p, size_t bytes) {
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e == cudaSuccess) {
        h->d2->allocs.push_back((void *)*p);
        h->dev_bytes += bytes;
    } else {
        *p = nullptr;
    }
    return e;
}

double feq9_host(double rho, double ux, double uy, int l) {
    const double cu = cx9(l) * ux + cy9(l) * uy, usq = ux * ux + uy * uy, cs2 = 1.0 / 3.0;
    return rho * w9d(l) *
           (1 + cu / cs2 + cu * cu / (2 * cs2 * cs2) - usq / (2 * cs2) + cu * cu * cu / (6 * cs2 * cs2 * cs2) -
            cu * usq / (2 * cs2 * cs2));
}

int face_priority2(int kind) {
    switch (kind) {
    case LBM_FACE_WALL: return 4;
    case LBM_FACE_INLET: return 3;
    case LBM_FACE_OUTLET_EQ: return 2;
    case LBM_FACE_OUTLET_ZG: return 1;
    }
    return 0;
}

// Boundary classes of the four faces: as for D3Q19 (a link crossing several
// ghost faces takes the highest-priority kind; a cell's wall velocity is the
// mean over its moving wall neighbours, Determine_Wall_Velocity,
// lbm.cpp:941-962).
// lface (optional): for every class and link whose source is a wall, the
// face that wall belongs to; -1 for the other links.
void build_classes2(const lbm_config &c, const Params2 &P, Class2 out[16], double uwall_out[16][2],
                    int (*lface)[Q9] = nullptr) {
    for (int cls = 0; cls < 16; cls++) {
        Class2 e;
        memset(&e, 0, sizeof(e));
        auto crossed = [&](int dx, int dy, int fs[2]) {
            int k = 0;
            if (!(P.periodic & 1)) {
                if (dx < 0 && (cls & 1)) fs[k++] = 0;
                if (dx > 0 && (cls & 2)) fs[k++] = 1;
            }
            if (!(P.periodic & 2)) {
                if (dy < 0 && (cls & 4)) fs[k++] = 2;
                if (dy > 0 && (cls & 8)) fs[k++] = 3;
            }
            return k;
        };
        auto resolve = [&](const int *fs, int k, double uw[2]) {
            int best = -1, bp = -1;
            for (int i = 0; i < k; i++) {
                const int p = face_priority2(c.faces[fs[i]].kind);
                if (p > bp) {
                    bp = p;
                    best = fs[i];
                }
            }
            uw[0] = uw[1] = 0.0;
            if (best >= 0 && c.faces[best].kind == LBM_FACE_WALL)
                for (int i = 0; i < k; i++) {
                    const lbm_face &F = c.faces[fs[i]];
                    if (F.kind == LBM_FACE_WALL && (F.u[0] != 0 || F.u[1] != 0)) {
                        uw[0] = F.u[0];
                        uw[1] = F.u[1];
                    }
                }
            return best;
        };
        double uwall[2] = {0, 0};
        int num = 0;
        for (int l = 0; l < Q9; l++) {
            int fs[2];
            const int k = crossed(cx9(l), cy9(l), fs);
            if (!k) continue;
            double uw[2];
            const int fi = resolve(fs, k, uw);
            if (c.faces[fi].kind == LBM_FACE_WALL && (uw[0] != 0 || uw[1] != 0)) {
                uwall[0] += uw[0];
                uwall[1] += uw[1];
                num++;
            }
        }
        if (num) {
            uwall[0] /= num;
            uwall[1] /= num;
        }
        if (uwall_out) {
            uwall_out[cls][0] = uwall[0];
            uwall_out[cls][1] = uwall[1];
        }
        for (int l = 0; l < Q9; l++) {
            int fs[2];
            const int k = crossed(-cx9(l), -cy9(l), fs);
            if (!k) continue;
            double uw[2];
            const int fi = resolve(fs, k, uw);
            const lbm_face &F = c.faces[fi];
            if (lface) lface[cls][l] = F.kind == LBM_FACE_WALL ? fi : -1;
            if (F.kind == LBM_FACE_WALL) {
                e.bb |= 1u << l;
                // f_l = f*_opp(l) - 2 w (u_w . c_opp) / cs^2 (lbm.cpp:274)
                e.val[l] = (float)(6.0 * w9d(l) * (uwall[0] * cx9(l) + uwall[1] * cy9(l)));
            } else if (F.kind == LBM_FACE_INLET || F.kind == LBM_FACE_OUTLET_EQ) {
                e.eq |= 1u << l;
                e.val[l] = (float)(feq9_host(F.rho, F.u[0], F.u[1], l) - w9d(l));
            } else if (F.kind == LBM_FACE_OUTLET_ZG) {
                e.zg |= 1u << l;
            }
        }
        out[cls] = e;
    }
}

// The ENERGY tables.  The wall temperature of Determine_Wall_Temperature
// (lbm.cpp:965-981) is the mean T of a cell's solid neighbours, taken with
// the periodic modulo over the whole ghost-inclusive grid; it is evaluated on
// that grid for one cell of each boundary class.  Before the first MacroProp
// the walls hold their set-up T; after it, the sum of their initial g (never
// streamed): the mean set-up T of their own solid neighbours, which for a
// wall row wraps onto the opposite wall row.  Corner ghost cells take the T
// of their y face.
// Neumann and adiabatic walls: the kind of each wall link's face; a class
// with wall links of two kinds is refused (returns false).
bool build_energy2(const lbm_config &c, const Params2 &P, const double uwall[16][2], const double uwall_w[16][2],
                   const int lface[16][Q9], Energy2 &E) {
    const double cs2 = 1.0 / 3.0, tg = c.tau_g;
    memset(&E, 0, sizeof(E));
    E.inv_tau_g = (float)(1.0 / tg);
    E.tg_fac = (float)((tg - 0.5) / (cs2 * tg));
    E.inv_cp = (float)(1.0 / c.cp);
    E.two_nu = (float)(2.0 * cs2 * (c.tau - 0.5));
    E.s_fac = (float)(-1.0 / (2.0 * c.tau * cs2));
    E.T_ref = (float)c.T_init;
    const int gx = (P.periodic & 1) ? 0 : 1, gy = (P.periodic & 2) ? 0 : 1;
    const int RX = P.nx + 2 * gx, RY = P.ny + 2 * gy;
    std::vector<uint8_t> solid((size_t)RX * RY, 0);
    std::vector<double> T0((size_t)RX * RY, c.T_init), T1((size_t)RX * RY, c.T_init);
    auto at = [&](int i, int j) { return (size_t)i + (size_t)RX * j; };
    for (int j = 0; j < RY; j++)
        for (int i = 0; i < RX; i++) {
            int f = -1;
            if (gy && j == 0) f = 2;
            else if (gy && j == RY - 1) f = 3;
            else if (gx && i == 0) f = 0;
            else if (gx && i == RX - 1) f = 1;
            if (f >= 0) {
                solid[at(i, j)] = 1;
                T0[at(i, j)] = c.faces[f].T;
            }
        }
    auto mean_solid = [&](const std::vector<double> &Tf, int i, int j) {
        int num = 0;
        double sum = 0.0;
        for (int l = 0; l < Q9; l++) {
            const int in = (i + cx9(l) + RX) % RX, jn = (j + cy9(l) + RY) % RY;
            if (solid[at(in, jn)]) {
                sum += Tf[at(in, jn)];
                num++;
            }
        }
        return num ? sum / num : 0.0;
    };
    for (int j = 0; j < RY; j++)
        for (int i = 0; i < RX; i++)
            if (solid[at(i, j)]) T1[at(i, j)] = mean_solid(T0, i, j);
    for (int cls = 0; cls < 16; cls++) {
        const int x = (cls & 1) ? 0 : ((cls & 2) ? P.nx - 1 : P.nx / 2);
        const int y = (cls & 4) ? 0 : ((cls & 8) ? P.ny - 1 : P.ny / 2);
        const double t0 = mean_solid(T0, x + gx, y + gy), t1 = mean_solid(T1, x + gx, y + gy);
        E.tw[cls][0] = (float)t0;
        E.tw[cls][1] = (float)t1;
        E.dtw[cls][0] = (float)(t0 - c.T_init);
        E.dtw[cls][1] = (float)(t1 - c.T_init);
        uint32_t dir = 0, neu = 0, adi = 0;
        for (int l = 0; l < Q9; l++) {
            if (!((P.cls[cls].bb >> l) & 1u)) continue;
            const int kind = c.faces[lface[cls][l]].thermal_kind;
            if (kind == LBM_TWALL_DIRICHLET) dir |= 1u << l;
            else if (kind == LBM_TWALL_NEUMANN) neu |= 1u << l;
            else adi |= 1u << l;
        }
        // classes no cell has: a periodic axis's face bits, or both faces of
        // an axis more than one cell long
        const bool occurs = !(((P.periodic & 1) && (cls & 3)) || ((P.periodic & 2) && (cls & 12)) ||
                              ((cls & 3) == 3 && P.nx > 1) || ((cls & 12) == 12 && P.ny > 1));
        if (occurs && (dir != 0) + (neu != 0) + (adi != 0) > 1) return false;
        E.dir[cls] = dir;
        E.neu[cls] = neu;
        E.adi[cls] = adi;
        if (neu) {
            // the normal: the mean direction of the wall links (the reference's
            // cdotn_pos, not normalised)
            double n0 = 0.0, n1 = 0.0;
            int np = 0;
            for (int l = 0; l < Q9; l++)
                if ((neu >> l) & 1u) {
                    n0 += cx9(l);
                    n1 += cy9(l);
                    np++;
                }
            n0 /= np;
            n1 /= np;
            const double u0 = uwall[cls][0], u1 = uwall[cls][1], uu = u0 * u0 + u1 * u1;
            double nk = 0.0, nd = 0.0;
            for (int l = 0; l < Q9; l++) {
                const double cn = cx9(l) * n0 + cy9(l) * n1;
                E.cn[cls][l] = (float)cn;
                const double uc = u0 * cx9(l) + u1 * cy9(l);
                if ((neu >> l) & 1u) {
                    nd += w9d(l) * (1 + uc / cs2 + pow(uc, 2) / (2 * cs2 * cs2) - uu / (2 * cs2) +
                                    pow(uc, 3) / (6 * pow(cs2, 3)) - uc * uu / (2 * cs2 * cs2)) *
                          cn;
                    // the g of link l: w rho T_w P2 of the solid direction -c_l
                    E.nq[cls][l] = (float)(1 - uc / cs2 + pow(uc, 2) / (2 * cs2 * cs2) - uu / (2 * cs2));
                } else {
                    nk += w9d(l) * cn;
                }
            }
            E.nk[cls] = (float)nk;
            E.nd[cls] = (float)nd;
        }
        for (int w = 0; w < 2; w++) {
            const double uwx = w ? uwall_w[cls][0] : uwall[cls][0], uwy = w ? uwall_w[cls][1] : uwall[cls][1];
            const double usq = uwx * uwx + uwy * uwy;
            for (int l = 0; l < Q9; l++) {
                // geq of the outgoing direction opp(l) (lbm.cpp:277-279)
                const double cu = -(cx9(l) * uwx + cy9(l) * uwy);
                const float v = (float)(cu / cs2 + cu * cu / (2 * cs2 * cs2) - usq / (2 * cs2) +
                                        cu * cu * cu / (6 * cs2 * cs2 * cs2) - cu * usq / (2 * cs2 * cs2));
                if (w) E.pm1_w[cls][l] = v;
                else E.pm1[cls][l] = v;
            }
        }
    }
    return true;
}

// The two launches of a D2Q9 step (collide-stream, IBM pass) go out with
// programmatic stream serialization: each launch is processed while its
// predecessor runs and its grid waits at cudaGridDependencySynchronize.
cudaLaunchConfig_t pdl_config2(dim3 grid, dim3 block, size_t smem, cudaStream_t s, cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t c = {};
    c.gridDim = grid;
    c.blockDim = block;
    c.dynamicSmemBytes = smem;
    c.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = attr;
    c.numAttrs = 1;
    return c;
}

// The streaming of step s (the gather of the launch made with s steps done)
// sees the walls moving at F/2 from s = 3 on when wall_force is set: the
// walls' force is set by the first MacroProp and enters their velocity at
// the second.
int wall_drift(const lbm_handle *h, int gather) { return (h->cfg.wall_force && gather && h->steps >= 3) ? 1 : 0; }

cudaError_t launch_energy2d(lbm_handle *h, int gather, float *mom, int export_only) {
    lbm2d *d = h->d2;
    const dim3 block(d->tx, d->ty);
    const dim3 grid((d->P.nx + d->tx - 1) / d->tx, (d->P.ny + d->ty - 1) / d->ty);
    const void *A = d->f[d->cur];
    void *B = d->f[1 - d->cur];
    const float *GA = d->g[d->cur];
    float *GB = d->g[1 - d->cur];
    const int first = gather && h->steps == 1 ? 1 : 0;
    const int drift = wall_drift(h, gather);
    const bool forced = d->P.forced != 0;
#define L2D_ENERGY(T)                                                                                           \
    if (forced)                                                                                               \
        k_energy2d<T, true><<<grid, block, 0, h->s>>>((const T *)A, (T *)B, GA, GB, d->P, d->E,                 \
                                                     d->st, d->aux, mom, gather, first, export_only, drift);   \
    else                                                                                                      \
        k_energy2d<T, false><<<grid, block, 0, h->s>>>((const T *)A, (T *)B, GA, GB, d->P,                      \
                                                      d->E, d->st, d->aux, mom, gather, first, export_only,    \
                                                      drift);
    L2D_ENERGY(float)
#undef L2D_ENERGY
    return cudaGetLastError();
}

cudaError_t launch_step2d(lbm_handle *h, int gather, float *mom, int export_only, int region = 0,
                          cudaStream_t stream = nullptr) {
    lbm2d *d = h->d2;
    if (d->energy) return launch_energy2d(h, gather, mom, export_only);
    const dim3 block(d->tx, d->ty);
    const int gw = region == 2 ? d->nbox.z : d->P.nx, gh = region == 2 ? d->nbox.w : d->P.ny;
    const dim3 grid((gw + d->tx - 1) / d->tx, (gh + d->ty - 1) / d->ty);
    const int4 nbx = d->nbox;
    const void *A = d->f[d->cur];
    void *B = d->f[1 - d->cur];
    const bool forced = d->P.forced != 0, solid = d->P.links != nullptr;
    const int drift = wall_drift(h, gather);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t lc = pdl_config2(grid, block, 0, region ? stream : h->s, attr);
    // the split launches follow event waits: plain launches
    if (region) lc.numAttrs = 0;
    cudaError_t e = cudaSuccess;
#define L2D_LAUNCH(T, FO, SO)                                                                                  \
    e = cudaLaunchKernelEx(&lc, k_step2d<T, FO, SO>, (const T *)A, (T *)B, d->P, d->st, mom, d->band, gather, \
                           export_only, drift, region, nbx)
#define L2D_STEP(T)                                                                                             \
    if (solid) {                                                                                              \
        if (forced) L2D_LAUNCH(T, true, true);                                                                \
        else L2D_LAUNCH(T, false, true);                                                                      \
    } else {                                                                                                  \
        if (forced) L2D_LAUNCH(T, true, false);                                                               \
        else L2D_LAUNCH(T, false, false);                                                                     \
    }
    switch (h->cfg.storage) {
    case LBM_STORE_F16: L2D_STEP(__half) break;
    case LBM_STORE_BF16: L2D_STEP(__nv_bfloat16) break;
    default: L2D_STEP(float) break;
    }
#undef L2D_STEP
#undef L2D_LAUNCH
    return e;
}

cudaError_t launch_ibm2d(lbm_handle *h, cudaStream_t stream) {
    lbm2d *d = h->d2;
    void *B = d->f[1 - d->cur];
    const size_t sm = d->ib.fast ? ibm2d_fast_smem_bytes(d->P.nb, d->ib.n)
                                 : (d->ib.smem ? ibm2d_smem_bytes(d->P.nb, d->ib.n) : 0);
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t c = pdl_config2(dim3(1), dim3(kIbmBlock), sm, stream, attr);
    switch (h->cfg.storage) {
    case LBM_STORE_F16: return cudaLaunchKernelEx(&c, k_ibm2d<__half>, (__half *)B, d->P, d->st, d->ib, d->band);
    case LBM_STORE_BF16:
        return cudaLaunchKernelEx(&c, k_ibm2d<__nv_bfloat16>, (__nv_bfloat16 *)B, d->P, d->st, d->ib, d->band);
    default: return cudaLaunchKernelEx(&c, k_ibm2d<float>, (float *)B, d->P, d->st, d->ib, d->band);
    }
}

// Opt the IBM kernel of this storage into the shared memory it needs.
cudaError_t ibm2d_smem_setup(int storage, size_t bytes) {
    switch (storage) {
    case LBM_STORE_F16:
        return cudaFuncSetAttribute(k_ibm2d<__half>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    case LBM_STORE_BF16:
        return cudaFuncSetAttribute(k_ibm2d<__nv_bfloat16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    default: return cudaFuncSetAttribute(k_ibm2d<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    }
}

// One reference iteration.
cudaError_t enqueue_step2d(lbm_handle *h) {
    lbm2d *d = h->d2;
    const int gather = h->steps == 0 ? 0 : 1;
    cudaError_t e = cudaSuccess;
    if (d->ibm) {
        // markers of the step (a moving body; a fixed one needs its nearest
        // nodes once) and, for the added mass of a moving body, the inside mask
        const bool moving = d->ib.motion != LBM_MOTION_FIXED;
        if (moving || (h->steps == 0 && d->ib.rho_nearest)) {
            const unsigned blocks = (unsigned)((d->ib.n * 32 + kMoveBlock - 1) / kMoveBlock);
            k_move2d<<<blocks, kMoveBlock, 0, h->s>>>(d->st, d->ib, d->P);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess && moving && d->ib.added_mass) {
            const unsigned blocks = (unsigned)((d->P.nb + kMoveBlock - 1) / kMoveBlock);
            k_inside2d<<<blocks, kMoveBlock, 0, h->s>>>(d->st, d->ib, d->P);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && d->overlap && gather) {
        // second stream: the near box (after the previous step's far cells)
        // and the IBM pass; this stream: the far cells, after the near box
        // (they read the previous state only) and beside the IBM pass
        e = cudaStreamWaitEvent(d->s2, d->ev_far, 0);
        if (e == cudaSuccess) e = launch_step2d(h, gather, nullptr, 0, 2, d->s2);
        if (e == cudaSuccess) e = cudaEventRecord(d->ev_near, d->s2);
        if (e == cudaSuccess) e = launch_ibm2d(h, d->s2);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(h->s, d->ev_near, 0);
        if (e == cudaSuccess) e = launch_step2d(h, gather, nullptr, 0, 1, h->s);
        if (e == cudaSuccess) e = cudaEventRecord(d->ev_far, h->s);
    } else {
        if (e == cudaSuccess) e = launch_step2d(h, gather, nullptr, 0);
        if (e == cudaSuccess && d->ibm) e = launch_ibm2d(h, h->s);
        if (e == cudaSuccess && d->overlap) e = cudaEventRecord(d->ev_far, h->s);
    }
    d->cur = 1 - d->cur;
    h->steps++;
    return e;
}

// A run of steps on the split streams starts from this stream's work and
// ends with the second stream joined back into it.
cudaError_t seq_begin2d(lbm_handle *h) {
    lbm2d *d = h->d2;
    return d->overlap ? cudaEventRecord(d->ev_far, h->s) : cudaSuccess;
}
cudaError_t seq_end2d(lbm_handle *h) {
    lbm2d *d = h->d2;
    if (!d->overlap) return cudaSuccess;
    cudaError_t e = cudaEventRecord(d->ev_join, d->s2);
    return e == cudaSuccess ? cudaStreamWaitEvent(h->s, d->ev_join, 0) : e;
}

// Whether the split applies: a fixed IBM body on plain cells whose near box
// (the IBM box of the step and one cell around it) lies inside the lattice,
// so that no periodic wrap reaches it, unless the configuration asks for the
// serial order (ibm_overlap < 0).  The box is read back once.
lbm_status decide_overlap2d(lbm_handle *h) {
    lbm2d *d = h->d2;
    if (d->overlap_known) return LBM_OK;
    d->overlap = false;
    if (d->ibm && d->ib.motion == LBM_MOTION_FIXED && !d->links && !d->energy && h->cfg.ibm_overlap >= 0) {
        State2 st;
        CK2(cudaStreamSynchronize(h->s));
        CK2(cudaMemcpy(&st, d->st, sizeof(State2), cudaMemcpyDeviceToHost));
        const int4 nb = make_int4(st.box_lo[0] - 1, st.box_lo[1] - 1, st.box_w + 2, st.box_h + 2);
        if (nb.x >= 0 && nb.y >= 0 && nb.x + nb.z <= d->P.nx && nb.y + nb.w <= d->P.ny && st.box_w > 0 &&
            st.box_h > 0) {
            if (!d->s2) {
                int lo = 0, hi = 0;
                CK2(cudaDeviceGetStreamPriorityRange(&lo, &hi));
                CK2(cudaStreamCreateWithPriority(&d->s2, cudaStreamNonBlocking, hi));
                CK2(cudaEventCreateWithFlags(&d->ev_far, cudaEventDisableTiming));
                CK2(cudaEventCreateWithFlags(&d->ev_near, cudaEventDisableTiming));
                CK2(cudaEventCreateWithFlags(&d->ev_join, cudaEventDisableTiming));
            }
            d->nbox = nb;
            d->overlap = true;
        }
    }
    d->overlap_known = true;
    return LBM_OK;
}

}  // namespace

lbm_status l2d_create(lbm_handle *h) {
    const lbm_config &c = h->cfg;
    if (c.nz != 1) return f2(LBM_ERR_INVALID, "create: a D2Q9 configuration has nz = 1");
    if (c.thermal != LBM_THERMAL_NONE && c.thermal != LBM_THERMAL_ENERGY)
        return f2(LBM_ERR_UNSUPPORTED, "create: D2Q9 handles take the ENERGY model (thermal = 2), not D3Q7");
    if (c.thermal == LBM_THERMAL_ENERGY) {
        if (!(c.cp > 0)) return f2(LBM_ERR_INVALID, "create: ENERGY needs cp > 0");
        if (c.storage != LBM_STORE_F32)
            return f2(LBM_ERR_UNSUPPORTED, "create: ENERGY handles store f in FP32 (T = sum g integrates every "
                                           "error of rho through geq = rho w T)");
        if (c.gbeta[0] != 0 || c.gbeta[1] != 0 || c.gbeta[2] != 0)
            return f2(LBM_ERR_UNSUPPORTED, "create: no buoyancy on ENERGY handles");
        for (int f = 0; f < 4; f++) {
            const lbm_face &F = c.faces[f];
            if (F.kind == LBM_FACE_PERIODIC) continue;
            if (F.kind != LBM_FACE_WALL || F.thermal_kind < LBM_TWALL_ADIABATIC ||
                F.thermal_kind > LBM_TWALL_NEUMANN)
                return f2(LBM_ERR_UNSUPPORTED, "create: ENERGY faces are periodic or walls (face " +
                                                   std::to_string(f) + ")");
        }
    }
    for (int a = 0; a < 2; a++) {
        const bool p0 = c.faces[2 * a].kind == LBM_FACE_PERIODIC, p1 = c.faces[2 * a + 1].kind == LBM_FACE_PERIODIC;
        if (p0 != p1) return f2(LBM_ERR_INVALID, "create: a periodic axis needs both faces periodic");
    }
    h->d2 = new lbm2d();
    lbm2d *d = h->d2;
    Params2 &P = d->P;
    memset(&P, 0, sizeof(P));
    P.nx = c.nx;
    P.ny = c.ny;
    P.N = (long long)c.nx * c.ny;
    P.S = ((P.N + 2LL * c.nx + 64 + 255) / 256) * 256;
    P.omega = (float)(1.0 / c.tau);
    P.body[0] = (float)c.body_force[0];
    P.body[1] = (float)c.body_force[1];
    P.forced = (c.body_force[0] != 0 || c.body_force[1] != 0) ? 1 : 0;
    for (int a = 0; a < 2; a++)
        if (c.faces[2 * a].kind == LBM_FACE_PERIODIC) P.periodic |= 1 << a;
    for (int l = 0; l < Q9; l++) P.pofs[l] = -(cx9(l) + c.nx * cy9(l));
    double uwall[16][2], uwall_w[16][2];
    int lface[16][Q9];
    for (int cls = 0; cls < 16; cls++)
        for (int l = 0; l < Q9; l++) lface[cls][l] = -1;
    build_classes2(c, P, P.cls, uwall, lface);
    {
        // the walls as seen from the third streaming on under wall_force:
        // their MacroProp velocity u_w + F / (2 rho_w), rho_w = 1
        lbm_config cw = c;
        for (int f = 0; f < 4; f++)
            if (c.wall_force && cw.faces[f].kind == LBM_FACE_WALL)
                for (int a = 0; a < 2; a++) cw.faces[f].u[a] += 0.5 * c.body_force[a];
        build_classes2(cw, P, P.cls_w, uwall_w);
    }
    d->energy = c.thermal == LBM_THERMAL_ENERGY;
    bool walls_kept = false;  // Neumann or adiabatic walls: the kept values
    if (d->energy) {
        if (!build_energy2(c, P, uwall, uwall_w, lface, d->E))
            return f2(LBM_ERR_UNSUPPORTED, "create: a cell next to walls of two thermal kinds (ENERGY)");
        for (int cls = 0; cls < 16; cls++) walls_kept = walls_kept || d->E.neu[cls] || d->E.adi[cls];
        if (walls_kept && c.wall_force)
            return f2(LBM_ERR_UNSUPPORTED, "create: Neumann or adiabatic walls with wall_force (ENERGY)");
    }
    h->esize = c.storage == LBM_STORE_F32 ? 4 : 2;
    if (c.graph_steps > 0) d->gsteps = c.graph_steps + (c.graph_steps & 1);
    if (c.graph_steps < 0) d->gsteps = 0;
    d->tx = c.block_x > 0 ? ((c.block_x + 31) / 32) * 32 : (c.nx >= 128 ? 128 : (c.nx >= 64 ? 64 : 32));
    // ENERGY steps (64 registers) ran 4 % faster in 128-thread blocks on a
    // 2048x1024 channel (33.0 k against 31.7 k MLUPS); the isothermal step is
    // indifferent between 128 and 256
    const int threads = c.thermal == LBM_THERMAL_ENERGY ? 128 : 256;
    d->ty = c.block_y > 0 ? c.block_y : std::max(1, threads / d->tx);
    CK2(cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking));
    for (int i = 0; i < 2; i++) CK2(alloc2(h, &d->f[i], (size_t)Q9 * P.S * h->esize));
    if (d->energy) {
        for (int i = 0; i < 2; i++) CK2(alloc2(h, &d->g[i], (size_t)Q9 * P.S * sizeof(float)));
        CK2(alloc2(h, &d->aux, (size_t)P.N * sizeof(float4)));
        if (walls_kept) CK2(alloc2(h, &d->E.gold, (size_t)Q9 * P.S * sizeof(float)));
    }
    // moments: rho, ux, uy (ENERGY: and T, qx, qy)
    CK2(alloc2(h, &d->mom, (size_t)(d->energy ? 6 : 3) * P.N * sizeof(float)));
    CK2(alloc2(h, &d->st, sizeof(State2)));
    CK2(alloc2(h, &d->hist, (size_t)d->hist_cap * 4 * sizeof(double)));
    State2 s0;
    memset(&s0, 0, sizeof(s0));
    s0.hist_cap = d->hist_cap;
    CK2(cudaMemcpyAsync(d->st, &s0, sizeof(s0), cudaMemcpyHostToDevice, h->s));
    CK2(cudaMemsetAsync(d->hist, 0, (size_t)d->hist_cap * 4 * sizeof(double), h->s));
    CK2(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

void l2d_free(lbm_handle *h) {
    lbm2d *d = h->d2;
    if (!d) return;
    for (int i = 0; i < 2; i++)
        if (d->gexec[i]) cudaGraphExecDestroy(d->gexec[i]);
    if (d->s2) {
        cudaStreamSynchronize(d->s2);
        cudaStreamDestroy(d->s2);
    }
    for (cudaEvent_t ev : {d->ev_far, d->ev_near, d->ev_join})
        if (ev) cudaEventDestroy(ev);
    for (void *p : d->allocs) cudaFree(p);
    if (d->fstage) cudaFreeHost(d->fstage);
    delete d;
    h->d2 = nullptr;
}

lbm_status l2d_init(lbm_handle *h, const double *rho, const double *ux, const double *uy) {
    lbm2d *d = h->d2;
    const long long N = d->P.N;
    float *dfields = nullptr;
    if (rho) {
        std::vector<float> tmp((size_t)3 * N);
        for (long long c = 0; c < N; c++) {
            tmp[c] = (float)rho[c];
            tmp[N + c] = (float)ux[c];
            tmp[2 * N + c] = (float)uy[c];
        }
        // staged through the moment buffer (3N floats)
        CK2(cudaMemcpyAsync(d->mom, tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice, h->s));
        dfields = d->mom;
        CK2(cudaStreamSynchronize(h->s));
    }
    const int thr = 256;
    const unsigned blocks = (unsigned)((N + thr - 1) / thr);
    const float r0 = (float)h->cfg.rho0, u0 = (float)h->cfg.u0[0], v0 = (float)h->cfg.u0[1];
    switch (h->cfg.storage) {
    case LBM_STORE_F16: k_init2d<__half><<<blocks, thr, 0, h->s>>>((__half *)d->f[0], N, d->P.S, dfields, r0, u0, v0); break;
    case LBM_STORE_BF16:
        k_init2d<__nv_bfloat16><<<blocks, thr, 0, h->s>>>((__nv_bfloat16 *)d->f[0], N, d->P.S, dfields, r0, u0, v0);
        break;
    default: k_init2d<float><<<blocks, thr, 0, h->s>>>((float *)d->f[0], N, d->P.S, dfields, r0, u0, v0); break;
    }
    CK2(cudaGetLastError());
    // solid cells are never written by a step: both buffers hold their state
    if (d->links) CK2(cudaMemcpyAsync(d->f[1], d->f[0], (size_t)Q9 * d->P.S * h->esize, cudaMemcpyDeviceToDevice, h->s));
    if (d->energy) {
        k_init_energy2d<<<blocks, thr, 0, h->s>>>(d->g[0], d->aux, N, d->P.S, dfields, r0, u0, v0, d->E.T_ref);
        CK2(cudaGetLastError());
    }
    CK2(cudaStreamSynchronize(h->s));
    d->cur = 0;
    h->steps = 0;
    h->inited = true;
    for (int i = 0; i < 2; i++) {
        if (!d->gexec[i]) continue;
        cudaGraphExecDestroy(d->gexec[i]);
        d->gexec[i] = nullptr;
    }
    d->overlap_known = false;
    return LBM_OK;
}

lbm_status l2d_set_markers(lbm_handle *h, const lbm_ibm_config *ic, const double *xyz, const double *dsw) {
    lbm2d *d = h->d2;
    if (d->ibm) return f2(LBM_ERR_STATE, "set_markers: markers already set");
    if (h->details)
        return f2(LBM_ERR_UNSUPPORTED, "set_markers: not on a D2Q9 handle in MORE_DETAILS mode (the reference's IBM "
                                       "loop never calls MacroProp, which forms the details)");
    if (d->energy) return f2(LBM_ERR_UNSUPPORTED, "set_markers: no immersed body on ENERGY handles");
    if (d->links) return f2(LBM_ERR_UNSUPPORTED, "set_markers: a D2Q9 handle takes solid cells or markers, not both");
    if (h->steps > 0) return f2(LBM_ERR_STATE, "set_markers: call before the first step");
    const int n = ic->n_markers;
    if (n < 1 || !xyz || !dsw) return f2(LBM_ERR_INVALID, "set_markers: bad markers");
    if (ic->free_body || ic->thermal) return f2(LBM_ERR_UNSUPPORTED, "set_markers: D2Q9 bodies are fixed or prescribed");
    if (ic->scheme == 0 && ic->m_max < 1) return f2(LBM_ERR_INVALID, "set_markers: m_max must be >= 1");
    if (ic->motion < LBM_MOTION_FIXED || ic->motion > LBM_MOTION_TRANSVERSE_OSC)
        return f2(LBM_ERR_INVALID, "set_markers: unknown motion");
    if (!(ic->radius > 0)) return f2(LBM_ERR_INVALID, "set_markers: radius must be positive");
    d->ic = *ic;
    Params2 &P = d->P;
    // the box [floor(c - D), ceil(c + D)] spans at most 2D + 2 nodes per axis
    const double D = 2.0 * ic->radius;
    P.bsx = std::min(P.nx, (int)std::ceil(2.0 * D) + 3);
    P.bsy = std::min(P.ny, (int)std::ceil(2.0 * D) + 3);
    P.nb = (long long)P.bsx * P.bsy;
    P.band_on = 1;
    Ibm2 &ib = d->ib;
    memset(&ib, 0, sizeof(ib));
    ib.n = n;
    ib.m_max = ic->m_max;
    ib.lit_sign = ic->literal_sign;
    ib.rho_nearest = ic->rho_nearest;
    ib.added_mass = ic->added_mass;
    ib.motion = ic->motion;
    ib.scheme = ic->scheme;
    ib.Dbox = D;
    ib.vsolid = ic->volume;
    ib.amp = ic->motion_amp;
    ib.freq = ic->motion_freq;
    for (int a = 0; a < 3; a++) ib.vconst[a] = ic->velocity[a];
    CK2(alloc2(h, &d->band, (size_t)5 * P.nb * sizeof(float)));
    CK2(alloc2(h, &ib.pos, (size_t)3 * n * sizeof(double)));
    double *nrm = nullptr, *dsd = nullptr;
    CK2(alloc2(h, &nrm, (size_t)3 * n * sizeof(double)));
    CK2(alloc2(h, &dsd, (size_t)n * sizeof(double)));
    ib.nrm = nrm;
    ib.dsw = dsd;
    CK2(alloc2(h, &ib.qnear, (size_t)n * sizeof(int)));
    CK2(alloc2(h, &ib.inside, (size_t)P.nb));
    CK2(alloc2(h, &ib.boxF, (size_t)4 * P.nb * sizeof(float)));
    CK2(cudaMemsetAsync(ib.boxF, 0, (size_t)4 * P.nb * sizeof(float), h->s));
    CK2(alloc2(h, &ib.fs, (size_t)2 * n * sizeof(float)));
    CK2(alloc2(h, &ib.rhom, (size_t)n * sizeof(float)));
    CK2(alloc2(h, &ib.s0, (size_t)2 * n * sizeof(int)));
    CK2(alloc2(h, &ib.swt, (size_t)16 * n * sizeof(float)));
    CK2(alloc2(h, &ib.cnt, (size_t)P.nb * sizeof(int)));
    CK2(alloc2(h, &ib.off, (size_t)P.nb * sizeof(int)));
    CK2(alloc2(h, &ib.lm, (size_t)16 * n * sizeof(int)));
    CK2(alloc2(h, &ib.lw, (size_t)16 * n * sizeof(float)));
    ib.hist = d->hist;
    // the pass's working set in shared memory when it fits
    const size_t sm = ibm2d_smem_bytes(P.nb, n);
    int dev = 0, optin = 0;
    CK2(cudaGetDevice(&dev));
    CK2(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    ib.smem = sm + 1024 <= (size_t)optin ? 1 : 0;
    const size_t smf = ibm2d_fast_smem_bytes(P.nb, n);
    ib.fast = (n <= kIbmBlock && P.nb <= (long long)kFastNodes * kIbmBlock && smf + 1024 <= (size_t)optin) ? 1 : 0;
    const size_t smax = std::max(ib.smem ? sm : (size_t)0, ib.fast ? smf : (size_t)0);
    if (smax > 0) CK2(ibm2d_smem_setup(h->cfg.storage, smax));
    CK2(cudaMemcpyAsync(ib.pos, xyz, (size_t)3 * n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    CK2(cudaMemcpyAsync(dsd, dsw, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    CK2(cudaMemsetAsync(nrm, 0, (size_t)3 * n * sizeof(double), h->s));
    CK2(cudaMemsetAsync(d->band, 0, (size_t)5 * P.nb * sizeof(float), h->s));
    // V_CM starts at zero (main.cpp: double V_CM[3] = {0,0,0}); the centre
    // is the given one
    State2 s0;
    CK2(cudaMemcpyAsync(&s0, d->st, sizeof(s0), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    for (int a = 0; a < 3; a++) {
        s0.center[a] = ic->center[a];
        s0.V[a] = s0.Vold[a] = 0.0;
    }
    s0.lists_ok = 0;
    s0.ibm_step = 0;
    CK2(cudaMemcpyAsync(d->st, &s0, sizeof(s0), cudaMemcpyHostToDevice, h->s));
    CK2(cudaStreamSynchronize(h->s));
    d->ibm = true;
    d->kin_ready = false;
    for (int i = 0; i < 2; i++) {
        if (!d->gexec[i]) continue;
        cudaGraphExecDestroy(d->gexec[i]);
        d->gexec[i] = nullptr;
    }
    d->overlap_known = false;
    return LBM_OK;
}

lbm_status l2d_set_normals(lbm_handle *h, const double *nxyz) {
    lbm2d *d = h->d2;
    if (!d->ibm) return f2(LBM_ERR_STATE, "set_marker_normals: call lbmgpu_set_markers first");
    CK2(cudaMemcpyAsync((void *)d->ib.nrm, nxyz, (size_t)3 * d->ib.n * sizeof(double), cudaMemcpyHostToDevice,
                        h->s));
    CK2(cudaStreamSynchronize(h->s));
    d->normals = true;
    return LBM_OK;
}

lbm_status l2d_step(lbm_handle *h, int nsteps) {
    lbm2d *d = h->d2;
    if (!h->inited) return f2(LBM_ERR_STATE, "step: call lbmgpu_init first");
    if (nsteps < 0) return f2(LBM_ERR_INVALID, "step: negative count");
    if (d->ibm && (d->ic.rho_nearest || d->ic.added_mass) && !d->normals)
        return f2(LBM_ERR_STATE, "step: the nearest-node density and the added mass need lbmgpu_set_marker_normals");
    if (d->ibm && !d->kin_ready) {
        // kinematics of reference step 1 (IBLBM's prelude)
        k_kin2d<<<1, 1, 0, h->s>>>(d->st, d->ib, d->P);
        CK2(cudaGetLastError());
        d->kin_ready = true;
    }
    if (d->ibm) {
        const lbm_status so = decide_overlap2d(h);
        if (so != LBM_OK) return so;
    }
    int left = nsteps;
    // the first step (no gather) and odd remainders run eagerly; whole
    // graphs of gsteps (even: the buffers return to the same parity) replay
    // (ENERGY: also the second, whose streaming takes the set-up wall T)
    // (wall_force: also until the walls' drift has set in, at the third)
    const long long eager = h->cfg.wall_force ? 3 : (d->energy ? 2 : 1);
    CK2(seq_begin2d(h));
    while (left > 0 && h->steps < eager) {
        CK2(enqueue_step2d(h));
        left--;
    }
    CK2(seq_end2d(h));
    if (d->gsteps > 0 && left >= d->gsteps) {
        cudaGraphExec_t &gx = d->gexec[d->cur];
        if (!gx) {
            cudaGraph_t g;
            const long long s0 = h->steps;
            const int c0 = d->cur;
            CK2(cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
            seq_begin2d(h);
            for (int i = 0; i < d->gsteps; i++) enqueue_step2d(h);
            seq_end2d(h);
            cudaError_t e = cudaStreamEndCapture(h->s, &g);
            h->steps = s0;
            d->cur = c0;
            CK2(e);
            e = cudaGraphInstantiate(&gx, g, 0);
            cudaGraphDestroy(g);
            CK2(e);
        }
        while (left >= d->gsteps) {
            CK2(cudaGraphLaunch(gx, h->s));
            h->steps += d->gsteps;
            left -= d->gsteps;
        }
    }
    CK2(seq_begin2d(h));
    while (left > 0) {
        CK2(enqueue_step2d(h));
        left--;
    }
    CK2(seq_end2d(h));
    return LBM_OK;
}

lbm_status l2d_export(lbm_handle *h) {
    lbm2d *d = h->d2;
    if (!h->inited) return f2(LBM_ERR_STATE, "download: call lbmgpu_init first");
    // gather-only pass over the current state (no collision, no store)
    const int gather = h->steps == 0 ? 0 : 1;
    CK2(launch_step2d(h, gather, d->mom, 1));
    return LBM_OK;
}

lbm_status l2d_download_f32(lbm_handle *h, int field, float *host) {
    lbm2d *d = h->d2;
    if (field < 0 || field > (d->energy ? 7 : 3)) return f2(LBM_ERR_INVALID, "download: bad field for a D2Q9 handle");
    const size_t N = (size_t)d->P.N;
    if (field == 3 || field == 7) {
        memset(host, 0, N * sizeof(float));
        return LBM_OK;
    }
    lbm_status s = l2d_export(h);
    if (s != LBM_OK) return s;
    // moment rows: rho, ux, uy (, T, qx, qy)
    const size_t row = field < 3 ? (size_t)field : (size_t)field - 1;
    CK2(cudaMemcpyAsync(host, d->mom + row * N, N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

lbm_status l2d_download_all_f32(lbm_handle *h, float *host) {
    lbm2d *d = h->d2;
    const size_t N = (size_t)d->P.N;
    lbm_status s = l2d_export(h);
    if (s != LBM_OK) return s;
    CK2(cudaMemcpyAsync(host, d->mom, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    if (d->energy) CK2(cudaMemcpyAsync(host + 4 * N, d->mom + 3 * N, N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    memset(host + 3 * N, 0, N * sizeof(float));
    return LBM_OK;
}

// The fields OutputVTK writes.  With markers they are those of the last
// IBLBM (lbm.cpp:1262-1285, 1342-1352): the moments of the populations the
// last step collided -- the buffer it pulled from, still intact -- and, in
// the box, the forced velocity and the force of that collision; without
// markers the moments of the current state.
lbm_status l2d_vtk_snapshot(lbm_handle *h, float *host, std::vector<float> &boxF, int box[4]) {
    lbm2d *d = h->d2;
    const size_t N = (size_t)d->P.N;
    if (!h->inited) return f2(LBM_ERR_STATE, "output_vtk: call lbmgpu_init first");
    if (d->ibm && h->steps > 0) {
        // the export pass of the last step: its source buffer and step count
        d->cur = 1 - d->cur;
        h->steps--;
        const cudaError_t e = launch_step2d(h, h->steps == 0 ? 0 : 1, d->mom, 1);
        d->cur = 1 - d->cur;
        h->steps++;
        CK2(e);
    } else {
        lbm_status s = l2d_export(h);
        if (s != LBM_OK) return s;
    }
    // the 3D moment layout: rho, u (3) [, T, q (3)]; uz and qz are zero
    CK2(cudaMemcpyAsync(host, d->mom, 3 * N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    if (d->energy) {
        CK2(cudaMemcpyAsync(host + 4 * N, d->mom + 3 * N, N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
        CK2(cudaMemcpyAsync(host + 5 * N, d->mom + 4 * N, 2 * N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    }
    box[0] = box[1] = box[2] = box[3] = 0;
    const size_t nb = (size_t)d->P.nb;
    if (d->ibm) {
        State2 st;
        boxF.resize(4 * nb);
        CK2(cudaMemcpyAsync(boxF.data(), d->ib.boxF, boxF.size() * sizeof(float), cudaMemcpyDeviceToHost, h->s));
        CK2(cudaMemcpyAsync(&st, d->st, sizeof(st), cudaMemcpyDeviceToHost, h->s));
        CK2(cudaStreamSynchronize(h->s));
        for (int k = 0; k < 4; k++) box[k] = st.fbox[k];
    }
    CK2(cudaStreamSynchronize(h->s));
    if (d->ibm && h->steps > 0) {
        for (int by = 0; by < box[3]; by++)
            for (int bx = 0; bx < box[2]; bx++) {
                const size_t o = (size_t)bx + (size_t)box[2] * by;
                const size_t cell = (size_t)(box[0] + bx) + (size_t)d->P.nx * (box[1] + by);
                host[N + cell] = boxF[2 * nb + o];
                host[2 * N + cell] = boxF[3 * nb + o];
            }
    }
    memset(host + 3 * N, 0, N * sizeof(float));
    if (d->energy) memset(host + 7 * N, 0, N * sizeof(float));
    return LBM_OK;
}

// Checkpoint regions: the populations of buffer src (and the ENERGY g and
// per-cell history), the device state (box, body, step, lists flag), the
// force history, and the markers' positions and nearest nodes (a fixed body
// finds them on its first step only).  The spreading lists are not saved:
// the restore marks them stale and the next pass rebuilds the same ones.
std::vector<l2d_region> l2d_checkpoint_regions(lbm_handle *h, int src) {
    lbm2d *d = h->d2;
    if (src < 0) src = d->cur;
    std::vector<l2d_region> r;
    const size_t es = h->cfg.storage == LBM_STORE_F32 ? 4 : 2;
    r.push_back({d->f[src], (size_t)Q9 * d->P.S * es, 1});
    if (d->energy) {
        r.push_back({d->g[src], (size_t)Q9 * d->P.S * sizeof(float), 1});
        r.push_back({d->aux, (size_t)d->P.N * sizeof(float4), 0});
        if (d->E.gold) r.push_back({d->E.gold, (size_t)Q9 * d->P.S * sizeof(float), 0});
    }
    r.push_back({d->st, sizeof(State2), 0});
    r.push_back({d->hist, (size_t)d->hist_cap * 4 * sizeof(double), 0});
    if (d->ibm) {
        r.push_back({d->ib.pos, (size_t)3 * d->ib.n * sizeof(double), 0});
        r.push_back({d->ib.qnear, (size_t)d->ib.n * sizeof(int), 0});
    }
    return r;
}

// lattice extents, storage, ENERGY, markers, solid cells, stride, history
void l2d_checkpoint_shape(lbm_handle *h, int shape[8]) {
    lbm2d *d = h->d2;
    shape[0] = d->P.nx;
    shape[1] = d->P.ny;
    shape[2] = h->cfg.storage;
    shape[3] = d->energy ? (d->E.gold ? 2 : 1) : 0;
    shape[4] = d->ibm ? d->ib.n : 0;
    shape[5] = d->links ? 1 : 0;
    shape[6] = (int)(d->P.S & 0x7fffffff);
    shape[7] = (int)d->hist_cap;
}

lbm_status l2d_checkpoint_restored(lbm_handle *h, long long steps) {
    lbm2d *d = h->d2;
    d->cur = 0;
    h->steps = steps;
    h->inited = true;
    if (d->ibm) {
        // the lists are rebuilt by the next pass; the box of the next step is
        // in the restored state, or made by the step-1 kinematics
        const int zero = 0;
        CK2(cudaMemcpyAsync(reinterpret_cast<char *>(d->st) + offsetof(State2, lists_ok), &zero, sizeof(int),
                            cudaMemcpyHostToDevice, h->s));
        d->kin_ready = steps > 0;
    }
    for (int i = 0; i < 2; i++) {
        if (!d->gexec[i]) continue;
        cudaGraphExecDestroy(d->gexec[i]);
        d->gexec[i] = nullptr;
    }
    d->overlap_known = false;
    CK2(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

long long l2d_cells(lbm_handle *h) { return h->d2->P.N; }
float *l2d_moments(lbm_handle *h) { return h->d2->mom; }

// MORE_DETAILS of the current state (k_details2d) behind a moment export, on
// the handle's stream; fold != 0 folds a Sup_MacroProp sample.
cudaError_t l2d_details_async(lbm_handle *h, int fold, double told, double dt) {
    lbm2d *d = h->d2;
    if (!h->inited) return cudaErrorNotReady;
    const int gather = h->steps == 0 ? 0 : 1;
    cudaError_t e = launch_step2d(h, gather, d->mom, 1);
    if (e != cudaSuccess) return e;
    const float sfac = (float)(-(h->cfg.tau - 0.5) / h->cfg.tau);
    const int drift = wall_drift(h, gather);
    const dim3 block(d->tx, d->ty);
    const dim3 grid((d->P.nx + d->tx - 1) / d->tx, (d->P.ny + d->ty - 1) / d->ty);
    const void *A = d->f[d->cur];
    const bool solid = d->P.links != nullptr;
#define L2D_DET(T)                                                                                             \
    if (solid)                                                                                               \
        k_details2d<T, true><<<grid, block, 0, h->s>>>((const T *)A, d->P, d->mom, h->det, h->stats, sfac,     \
                                                       gather, drift, fold, told, dt);                        \
    else                                                                                                     \
        k_details2d<T, false><<<grid, block, 0, h->s>>>((const T *)A, d->P, d->mom, h->det, h->stats, sfac,    \
                                                        gather, drift, fold, told, dt);
    switch (h->cfg.storage) {
    case LBM_STORE_F16: L2D_DET(__half) break;
    case LBM_STORE_BF16: L2D_DET(__nv_bfloat16) break;
    default: L2D_DET(float) break;
    }
#undef L2D_DET
    return cudaGetLastError();
}

bool l2d_has_markers(lbm_handle *h) { return h->d2->ibm; }

int l2d_marker_count(lbm_handle *h) { return h->d2->ibm ? h->d2->ib.n : 0; }

// The last `take` rows of the force ring (drag, lift, 0, step) as the rows
// of lbmgpu_get_forces (Fx, Fy, 0, 0, 0, 0, 0, step), stored into pinned,
// device-mapped host memory: one launch and one synchronisation for a read
// the reference's loop makes every step, however long the ring.
__global__ void k_forces2d_out(const double *__restrict__ hist, long long cap, long long steps, long long take,
                               double *__restrict__ dst) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < take * 8;
         e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e & 7);
        // reference step steps - take + 1 + (e >> 3), 1-based
        const double *r = hist + 4 * ((steps - take + (e >> 3)) % cap);
        dst[e] = k < 2 ? r[k] : (k == 7 ? r[3] : 0.0);
    }
}

lbm_status l2d_get_forces(lbm_handle *h, double *out, int max_steps, int *n_out) {
    lbm2d *d = h->d2;
    if (!d->ibm) return f2(LBM_ERR_STATE, "get_forces: no markers set");
    const long long take = std::min<long long>(std::min<long long>(h->steps, d->hist_cap), max_steps);
    if (take > d->fstage_rows) {
        if (d->fstage) {
            CK2(cudaStreamSynchronize(h->s));
            CK2(cudaFreeHost(d->fstage));
            d->fstage = nullptr;
            d->fstage_rows = 0;
        }
        const long long cap = std::max<long long>(take, 64);
        CK2(cudaHostAlloc((void **)&d->fstage, (size_t)cap * 8 * sizeof(double), cudaHostAllocMapped));
        d->fstage_rows = cap;
    }
    if (take > 0) {
        double *dst = nullptr;
        CK2(cudaHostGetDevicePointer((void **)&dst, d->fstage, 0));
        const unsigned blocks = (unsigned)std::min<long long>((take * 8 + 255) / 256, 64);
        k_forces2d_out<<<blocks, 256, 0, h->s>>>(d->hist, d->hist_cap, h->steps, take, dst);
        CK2(cudaGetLastError());
    }
    CK2(cudaStreamSynchronize(h->s));
    if (take > 0) std::memcpy(out, d->fstage, (size_t)take * 8 * sizeof(double));
    if (n_out) *n_out = (int)take;
    return LBM_OK;
}

lbm_status l2d_get_markers(lbm_handle *h, double *xyz) {
    lbm2d *d = h->d2;
    if (!d->ibm) return f2(LBM_ERR_STATE, "get_markers: no markers set");
    CK2(cudaMemcpyAsync(xyz, d->ib.pos, (size_t)3 * d->ib.n * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

lbm_status l2d_get_body(lbm_handle *h, double out[9]) {
    lbm2d *d = h->d2;
    State2 s;
    CK2(cudaMemcpyAsync(&s, d->st, sizeof(s), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    for (int a = 0; a < 3; a++) {
        out[a] = s.center[a];
        out[3 + a] = s.V[a];
        out[6 + a] = 0.0;
    }
    return LBM_OK;
}

lbm_status l2d_set_solids(lbm_handle *h, const uint8_t *mask) {
    lbm2d *d = h->d2;
    if (h->inited) return f2(LBM_ERR_STATE, "set_solids: call before lbmgpu_init");
    if (d->links) return f2(LBM_ERR_STATE, "set_solids: solids already set");
    if (d->ibm) return f2(LBM_ERR_UNSUPPORTED, "set_solids: a D2Q9 handle takes solid cells or markers, not both");
    if (d->energy) return f2(LBM_ERR_UNSUPPORTED, "set_solids: no interior solids on ENERGY handles");
    const Params2 &P = d->P;
    std::vector<uint16_t> lk((size_t)P.N, 0);
    long long nsolid = 0;
    for (int y = 0; y < P.ny; y++)
        for (int x = 0; x < P.nx; x++) {
            const size_t c = (size_t)x + (size_t)P.nx * y;
            if (mask[c]) {
                lk[c] = (uint16_t)kSolidCell;
                nsolid++;
                continue;
            }
            for (int l = 1; l < Q9; l++) {
                int sx = x - cx9(l), sy = y - cy9(l);
                if (P.periodic & 1) sx = (sx + P.nx) % P.nx;
                if (P.periodic & 2) sy = (sy + P.ny) % P.ny;
                if (sx < 0 || sx >= P.nx || sy < 0 || sy >= P.ny) continue;
                if (mask[(size_t)sx + (size_t)P.nx * sy]) lk[c] |= (uint16_t)(1u << l);
            }
        }
    if (nsolid == 0) return LBM_OK;
    CK2(alloc2(h, &d->links, (size_t)P.N * sizeof(uint16_t)));
    CK2(alloc2(h, &d->mea_out, 4 * sizeof(double)));
    CK2(cudaMemcpyAsync(d->links, lk.data(), lk.size() * sizeof(uint16_t), cudaMemcpyHostToDevice, h->s));
    CK2(cudaStreamSynchronize(h->s));
    d->P.links = d->links;
    h->solids = true;
    return LBM_OK;
}

lbm_status l2d_thermal_moments(lbm_handle *h, const float **uy, const float **T, const uint16_t **links, long long *N) {
    lbm2d *d = h->d2;
    if (!d->energy) return f2(LBM_ERR_STATE, "nusselt: the handle has no temperature (ENERGY)");
    lbm_status s = l2d_export(h);
    if (s != LBM_OK) return s;
    *uy = d->mom + 2 * d->P.N;
    *T = d->mom + 3 * d->P.N;
    *links = d->links;
    *N = d->P.N;
    return LBM_OK;
}

lbm_status l2d_mea_box(lbm_handle *h, const int box[6], double out[3]) {
    lbm2d *d = h->d2;
    if (!d->links) return f2(LBM_ERR_STATE, "mea_box: no solid cells set");
    if (!h->inited) return f2(LBM_ERR_STATE, "mea_box: call lbmgpu_init first");
    const Params2 &P = d->P;
    // the reference's ghost-inclusive indices -> device cells (a periodic
    // axis has no ghost layer on the device); the computational layer k = 1
    out[0] = out[1] = out[2] = 0.0;
    if (box[4] > 1 || box[5] < 1) return LBM_OK;
    const int ox = (P.periodic & 1) ? 0 : 1, oy = (P.periodic & 2) ? 0 : 1;
    const int x0 = std::max(box[0] - ox, 0), x1 = std::min(box[1] - ox, P.nx - 1);
    const int y0 = std::max(box[2] - oy, 0), y1 = std::min(box[3] - oy, P.ny - 1);
    if (x0 > x1 || y0 > y1) return LBM_OK;
    const void *A = d->f[d->cur];
    const int drift = wall_drift(h, 1);
    switch (h->cfg.storage) {
    case LBM_STORE_F16:
        k_mea2d<__half><<<1, 256, 0, h->s>>>((const __half *)A, P, x0, x1, y0, y1, d->mea_out, drift);
        break;
    case LBM_STORE_BF16:
        k_mea2d<__nv_bfloat16><<<1, 256, 0, h->s>>>((const __nv_bfloat16 *)A, P, x0, x1, y0, y1, d->mea_out, drift);
        break;
    default: k_mea2d<float><<<1, 256, 0, h->s>>>((const float *)A, P, x0, x1, y0, y1, d->mea_out, drift); break;
    }
    CK2(cudaGetLastError());
    CK2(cudaMemcpyAsync(out, d->mea_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

lbm_status l2d_status(lbm_handle *h, uint32_t *flags) {
    lbm2d *d = h->d2;
    uint32_t v = 0;
    CK2(cudaMemcpyAsync(&v, &d->st->status, sizeof(v), cudaMemcpyDeviceToHost, h->s));
    CK2(cudaStreamSynchronize(h->s));
    *flags = v;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_config_from_types_2d(int nx, int ny, double tau, const uint8_t *types,
                                                  const double *rho, const double *ux, const double *uy,
                                                  lbm_config *out) {
    if (!types || !out || nx < 1 || ny < 1) return f2(LBM_ERR_INVALID, "config_from_types_2d: bad arguments");
    const int NX = nx + 2;
    auto at = [&](int i, int j) { return (size_t)i + (size_t)NX * j; };
    lbm_config c;
    memset(&c, 0, sizeof(c));
    c.tau = tau;
    c.rho0 = 1.0;
    c.lattice = LBM_LATTICE_D2Q9;
    // interior TYPE_S cells at rest are staircase bodies (lbmgpu_set_solids)
    for (int j = 1; j <= ny; j++)
        for (int i = 1; i <= nx; i++) {
            const int t = types[at(i, j)];
            if (t == 1 && ux && uy && (ux[at(i, j)] != 0 || uy[at(i, j)] != 0))
                return f2(LBM_ERR_UNSUPPORTED, "config_from_types_2d: moving interior solid cell");
            if (t != 0 && t != 1)
                return f2(LBM_ERR_UNSUPPORTED, "config_from_types_2d: non-fluid cell inside the domain");
        }
    int periodic_axis[2] = {0, 0};
    for (int f = 0; f < 4; f++) {
        const int a = f / 2, side = f % 2;
        const int lim = a == 0 ? ny : nx;
        int kind0 = -1;
        double st[3] = {0, 0, 0};
        for (int p = 1; p <= lim; p++) {
            const size_t id = a == 0 ? at(side ? nx + 1 : 0, p) : at(p, side ? ny + 1 : 0);
            const int t = types[id];
            const double s[3] = {rho ? rho[id] : 1.0, ux ? ux[id] : 0.0, uy ? uy[id] : 0.0};
            if (kind0 < 0) {
                kind0 = t;
                memcpy(st, s, sizeof(st));
            } else if (t != kind0 || memcmp(st, s, sizeof(st)) != 0) {
                return f2(LBM_ERR_UNSUPPORTED, "config_from_types_2d: face " + std::to_string(f) + " is not uniform");
            }
        }
        lbm_face &F = c.faces[f];
        F.rho = st[0];
        F.u[0] = st[1];
        F.u[1] = st[2];
        switch (kind0) {
        case 1: F.kind = LBM_FACE_WALL; break;
        case 3: F.kind = LBM_FACE_INLET; break;
        case 2: F.kind = LBM_FACE_OUTLET_EQ; break;
        case 0: F.kind = LBM_FACE_PERIODIC; periodic_axis[a]++; break;
        default:
            return f2(LBM_ERR_UNSUPPORTED, "config_from_types_2d: unsupported ghost type " + std::to_string(kind0));
        }
    }
    int dims[2] = {nx, ny};
    for (int a = 0; a < 2; a++) {
        if (periodic_axis[a] == 1) return f2(LBM_ERR_UNSUPPORTED, "config_from_types_2d: one-sided TYPE_F ghost face");
        if (periodic_axis[a] == 2) dims[a] += 2;  // the reference wraps over N+2 cells
    }
    c.faces[4].kind = c.faces[5].kind = LBM_FACE_PERIODIC;
    c.nx = dims[0];
    c.ny = dims[1];
    c.nz = 1;
    *out = c;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_config_energy_2d(lbm_config *cfg, int nx, int ny, const uint8_t *types,
                                              const uint8_t *types_energy, const double *T, double tau_g, double cp) {
    if (!cfg || !types || !types_energy || !T || nx < 1 || ny < 1)
        return f2(LBM_ERR_INVALID, "config_energy_2d: bad arguments");
    if (cfg->lattice != LBM_LATTICE_D2Q9) return f2(LBM_ERR_INVALID, "config_energy_2d: not a D2Q9 configuration");
    const int NX = nx + 2, NY = ny + 2;
    auto at = [&](int i, int j) { return (size_t)i + (size_t)NX * j; };
    // the fluid's set-up T (the periodic ghost layers included): uniform
    bool have = false;
    double Tf = 0.0;
    for (int j = 0; j < NY; j++)
        for (int i = 0; i < NX; i++) {
            if (types[at(i, j)] != 0) continue;
            if (!have) {
                Tf = T[at(i, j)];
                have = true;
            } else if (T[at(i, j)] != Tf) {
                return f2(LBM_ERR_UNSUPPORTED, "config_energy_2d: the fluid's set-up T is not uniform");
            }
        }
    if (!have) return f2(LBM_ERR_INVALID, "config_energy_2d: no fluid cell");
    for (int f = 0; f < 4; f++) {
        lbm_face &F = cfg->faces[f];
        if (F.kind == LBM_FACE_PERIODIC) continue;
        if (F.kind != LBM_FACE_WALL)
            return f2(LBM_ERR_UNSUPPORTED, "config_energy_2d: inlet/outlet faces are not supported with ENERGY");
        const int a = f / 2, side = f % 2;
        const int lim = a == 0 ? ny : nx;
        // type_Energy TYPE_T (6): Dirichlet; TYPE_Q (7): Neumann with the
        // reference's j_dot_n = 0 (LBM.h); any other: adiabatic
        int kind = LBM_TWALL_ADIABATIC;
        for (int p = 1; p <= lim; p++) {
            const size_t id = a == 0 ? at(side ? nx + 1 : 0, p) : at(p, side ? ny + 1 : 0);
            const int te = types_energy[id];
            const int k = te == 6 ? LBM_TWALL_DIRICHLET : (te == 7 ? LBM_TWALL_NEUMANN : LBM_TWALL_ADIABATIC);
            if (p == 1) kind = k;
            else if (k != kind)
                return f2(LBM_ERR_UNSUPPORTED,
                          "config_energy_2d: face " + std::to_string(f) + " mixes thermal wall types");
            if (p == 1) F.T = T[id];
            else if (T[id] != F.T)
                return f2(LBM_ERR_UNSUPPORTED, "config_energy_2d: face " + std::to_string(f) + " T is not uniform");
        }
        F.thermal_kind = kind;
    }
    cfg->thermal = LBM_THERMAL_ENERGY;
    cfg->tau_g = tau_g;
    cfg->cp = cp;
    cfg->T_init = Tf;
    return LBM_OK;
}
