// lbm_step.cuh -- per-cell pieces of the fused collide-stream step shared
// by the one-cell (k_step) and multi-cell (k_stepv) kernels: the pull of
// the 19 (+7) populations with the boundary-class rules, and the update
// (moments, IBM band hand-off or BGK + Guo collision).
#pragma once
#include "lbm_collide.cuh"
#include "lbm_device.cuh"

namespace lbmk {

// One link of the boundary-class path: bounce-back, face equilibrium, or a
// pull from the (wrapped, or zero-gradient clamped) source cell.
template <class T>
__device__ __forceinline__ float pull_link(const T *__restrict__ A, int l, int x, int y, int z, long long cell,
                                           const ClassEntry &ce, const StepParams &P) {
    if ((ce.bb >> l) & 1u) return St<T>::ld(A + opp(l) * P.S + cell) + ce.val[l];
    if ((ce.eq >> l) & 1u) return ce.val[l];
    int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
    // periodic axes wrap; a zero-gradient link then clamps the remaining
    // ghost coordinates onto the interior
    if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
    if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
    if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
    if ((ce.zg >> l) & 1u) {
        sx = min(max(sx, 0), P.nx - 1);
        sy = min(max(sy, 0), P.ny - 1);
        sz = min(max(sz, 0), P.nz - 1);
    }
    return St<T>::ld(A + l * P.S + sx + (long long)P.nx * (sy + (long long)P.ny * sz));
}

// Link k of the x-face table (XFix) for the cell at 32-bit index c.
template <class T>
__device__ __forceinline__ float xfix_link(const T *__restrict__ A, unsigned c, const XFix &xf, int k) {
    const float v = St<T>::ld(A + (c + xf.ofs[k]));
    return ((xf.eq >> k) & 1u) ? xf.add[k] : __fmaf_rn(xf.sgn[k], v, xf.add[k]);
}
template <class T>
__device__ __forceinline__ float xfix_heat(const T *__restrict__ G, unsigned c, const XFix &xf) {
    const float v = St<T>::ld(G + (c + xf.tofs));
    return xf.teq ? xf.tadd : __fmaf_rn(xf.tsgn, v, xf.tadd);
}

__device__ __forceinline__ int periodic_mask(const StepParams &P) {
    return ((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0) | ((P.periodic & 4) ? 48 : 0);
}

// Pull the 19 populations of one cell.  A warp whose lanes all lie in rows
// off the y/z faces takes the plain offsets; a lane on x = 0 or x = nx-1
// then redoes the five links that cross its x face with the boundary-class
// rule (xfix).  Any other warp takes the boundary-class path for every link.
template <class T>
__device__ __forceinline__ void gather_flow(const T *__restrict__ A, float f[Q], int x, int y, int z,
                                            long long cell, int raw_cls, bool valid, bool bwarp, int gather,
                                            const StepParams &P) {
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(A + l * P.S + cell) : 0.0f;
        return;
    }
    if (!bwarp) {
        const T *a = A + cell;
        if (P.idx32) {
            // idle lanes read a safe stencil instead of being predicated off
            const unsigned c = valid ? (unsigned)cell : P.safe_cell;
#pragma unroll
            for (int l = 0; l < Q; l++) f[l] = St<T>::ld(A + (c + P.pofs32[l]));
        } else {
#pragma unroll
            for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(a + P.pofs[l]) : 0.0f;
        }
        if (raw_cls & 3) {
            if (P.idx32) {
                // the x-face table: the same values, without per-link branches
                const unsigned c = (unsigned)cell;
                if (raw_cls & 1) {
#pragma unroll
                    for (int k = 0; k < 5; k++) f[xpl(k)] = xfix_link<T>(A, c, P.xf[0], k);
                }
                if (raw_cls & 2) {
#pragma unroll
                    for (int k = 0; k < 5; k++) f[xml(k)] = xfix_link<T>(A, c, P.xf[1], k);
                }
            } else {
                const ClassEntry &ce = P.cls[raw_cls & 3 & ~periodic_mask(P)];
#pragma unroll
                for (int l = 1; l < Q; l++) {
                    if (cx(l) > 0 && (raw_cls & 1)) f[l] = pull_link<T>(A, l, x, y, z, cell, ce, P);
                    if (cx(l) < 0 && (raw_cls & 2)) f[l] = pull_link<T>(A, l, x, y, z, cell, ce, P);
                }
            }
        }
        return;
    }
    const ClassEntry &ce = P.cls[raw_cls & ~periodic_mask(P)];
#pragma unroll
    for (int l = 0; l < Q; l++) f[l] = valid ? pull_link<T>(A, l, x, y, z, cell, ce, P) : 0.0f;
}

// One D3Q7 link of the boundary-class path: adiabatic or Dirichlet
// (anti-)bounce-back, face equilibrium, or a pull from the source cell.
template <class T>
__device__ __forceinline__ float pull_heat_link(const T *__restrict__ G, int l, int x, int y, int z, long long cell,
                                                const ClassEntry &ce, const StepParams &P) {
    if ((ce.bb >> l) & 1u) {
        const float own = St<T>::ld(G + opp(l) * P.S + cell);
        return ((ce.tdir >> l) & 1u) ? (-own + ce.tval[l]) : own;
    }
    if ((ce.eq >> l) & 1u) return ce.tval[l];
    int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
    if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
    if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
    if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
    if ((ce.zg >> l) & 1u) {
        sx = min(max(sx, 0), P.nx - 1);
        sy = min(max(sy, 0), P.ny - 1);
        sz = min(max(sz, 0), P.nz - 1);
    }
    return St<T>::ld(G + l * P.S + sx + (long long)P.nx * (sy + (long long)P.ny * sz));
}

// The D3Q7 temperature populations, with the same split as gather_flow.
template <class T>
__device__ __forceinline__ void gather_heat(const T *__restrict__ G, float g[QT], int x, int y, int z,
                                            long long cell, int raw_cls, bool valid, bool bwarp, int gather,
                                            const StepParams &P) {
    if (!gather) {
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = valid ? St<T>::ld(G + l * P.S + cell) : 0.0f;
        return;
    }
    if (!bwarp) {
        const T *a = G + cell;
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = valid ? St<T>::ld(a + P.pofs[l]) : 0.0f;
        if (raw_cls & 3) {
            if (P.idx32) {
                if (raw_cls & 1) g[1] = xfix_heat<T>(G, (unsigned)cell, P.xf[0]);
                if (raw_cls & 2) g[2] = xfix_heat<T>(G, (unsigned)cell, P.xf[1]);
            } else {
                const ClassEntry &ce = P.cls[raw_cls & 3 & ~periodic_mask(P)];
#pragma unroll
                for (int l = 1; l < QT; l++) {
                    if (cx(l) > 0 && (raw_cls & 1)) g[l] = pull_heat_link<T>(G, l, x, y, z, cell, ce, P);
                    if (cx(l) < 0 && (raw_cls & 2)) g[l] = pull_heat_link<T>(G, l, x, y, z, cell, ce, P);
                }
            }
        }
        return;
    }
    const ClassEntry &ce = P.cls[raw_cls & ~periodic_mask(P)];
#pragma unroll
    for (int l = 0; l < QT; l++) g[l] = valid ? pull_heat_link<T>(G, l, x, y, z, cell, ce, P) : 0.0f;
}

// Pull of a cell near interior solid cells (staircase bodies).  A link whose
// source cell is a solid bounces back the cell's own post-collision
// population of the opposite link (stationary wall: no velocity term); every
// other link follows the boundary-class rules.  A solid cell itself keeps its
// populations (read in place: its moments for the read-back).  mea gets the
// momentum exchange of the cell, sum over its solid links of
// (f*_l + f_opp(l)) c_l with f* the cell's post-collision and f the pulled
// populations (MEA_CD / MEA_CL, lbm.cpp:3085-3163; shifted storage adds
// 2 w_l).
template <class T, bool THERMAL>
__device__ __forceinline__ void gather_solid(const T *__restrict__ A, const T *__restrict__ G, float f[Q],
                                             float g[QT], int x, int y, int z, long long cell, int raw_cls,
                                             bool valid, bool solid_cell, int gather, const StepParams &P,
                                             float mea[3]) {
    mea[0] = mea[1] = mea[2] = 0.0f;
    if (!valid || !gather || solid_cell) {
#pragma unroll
        for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(A + l * P.S + cell) : 0.0f;
        if (THERMAL) {
#pragma unroll
            for (int l = 0; l < QT; l++) g[l] = valid ? St<T>::ld(G + l * P.S + cell) : 0.0f;
        }
        return;
    }
    const ClassEntry &ce = P.cls[raw_cls & ~periodic_mask(P)];
    uint32_t sl = 0;
#pragma unroll
    for (int l = 1; l < Q; l++) {
        int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
        if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
        if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
        if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
        const bool inside = (unsigned)sx < (unsigned)P.nx && (unsigned)sy < (unsigned)P.ny && (unsigned)sz < (unsigned)P.nz;
        if (inside && mask_bit(P.solid, sx + (long long)P.nx * (sy + (long long)P.ny * sz))) sl |= 1u << l;
    }
    f[0] = St<T>::ld(A + cell);
#pragma unroll
    for (int l = 1; l < Q; l++)
        f[l] = ((sl >> l) & 1u) ? St<T>::ld(A + opp(l) * P.S + cell) : pull_link<T>(A, l, x, y, z, cell, ce, P);
    if (THERMAL) {
        g[0] = St<T>::ld(G + cell);
#pragma unroll
        for (int l = 1; l < QT; l++)  // adiabatic bounce-back of the D3Q7 population on solid links
            g[l] = ((sl >> l) & 1u) ? St<T>::ld(G + opp(l) * P.S + cell) : pull_heat_link<T>(G, l, x, y, z, cell, ce, P);
    }
    if (P.mea != nullptr && sl) {
#pragma unroll
        for (int l = 1; l < Q; l++) {
            if (!((sl >> l) & 1u)) continue;
            const float t = St<T>::ld(A + l * P.S + cell) + f[opp(l)] + 2.0f * wf(l);
            mea[0] += t * cx(l);
            mea[1] += t * cy(l);
            mea[2] += t * cz(l);
        }
    }
}

// Moments, force and velocity of one cell (F = float) or of two neighbouring
// cells (F = float2): the part of the update every step kernel shares.
// Body force plus Boussinesq buoyancy F = Fb + gbeta (T - T0); velocity
// u = (j + hf F) / rho, hf = 1/2 once the populations have been streamed
// (MacroProp, lbm.cpp:677-679) and 0 before the first streaming, when the
// reference collides with the velocity stored at set-up (LBM::Init,
// lbm.cpp:31-57).
template <class F, bool THERMAL, bool FORCED>
__device__ __forceinline__ void cell_state(const F f[Q], const F g[QT], const StepParams &P, float hf, F &drho,
                                           F &ux, F &uy, F &uz, F &Fx, F &Fy, F &Fz, F &Tc) {
    using A = Ar<F>;
    F jx, jy, jz;
    moments_pairs(f, drho, jx, jy, jz);
    Fx = A::splat(P.body[0]);
    Fy = A::splat(P.body[1]);
    Fz = A::splat(P.body[2]);
    Tc = A::splat(0.0f);
    if constexpr (THERMAL) {
        Tc = heat_sum(g);
        const F dT = A::sub(Tc, A::splat(P.T0));
        Fx = A::fma(A::splat(P.gbeta[0]), dT, Fx);
        Fy = A::fma(A::splat(P.gbeta[1]), dT, Fy);
        Fz = A::fma(A::splat(P.gbeta[2]), dT, Fz);
    }
    const F inv = inv_one_plus(drho);
    if constexpr (FORCED) {
        const F h = A::splat(hf);
        ux = A::mul(A::fma(h, Fx, jx), inv);
        uy = A::mul(A::fma(h, Fy, jy), inv);
        uz = A::mul(A::fma(h, Fz, jz), inv);
    } else {
        ux = A::mul(jx, inv);
        uy = A::mul(jy, inv);
        uz = A::mul(jz, inv);
    }
}

// Everything after the gather of one cell except the stores: moments,
// optional moment output, then either the band hand-off (f, g keep the
// pre-collision populations; the unforced moments go to the band arrays) or
// the collision.  Returns whether f (and g) are to be stored for this cell.
template <class T, bool THERMAL, bool FORCED>
__device__ __forceinline__ bool update_cell(float f[Q], float g[QT], int x, int y, int z, long long cell, bool valid,
                                            int gather, int export_only, const StepParams &P,
                                            DevState *__restrict__ ds, float *__restrict__ mom,
                                            float *__restrict__ band, bool check_band, bool frozen = false) {
    const long long N = P.N;
    float drho, ux, uy, uz, Fx, Fy, Fz, Tc;
    cell_state<float, THERMAL, FORCED>(f, g, P, gather ? 0.5f : 0.0f, drho, ux, uy, uz, Fx, Fy, Fz, Tc);
    const float rho = __fadd_rn(1.0f, drho);
    // one status update per warp (every lane of the warp runs this): a
    // diverged solve would otherwise send an atomic from every cell
    const unsigned badw = __ballot_sync(0xffffffffu, valid && !(rho > 0.0f && rho < 100.0f));
    if (badw && (threadIdx.x & 31) == 0) raise_status(&ds->status, ST_RHO_RANGE);
    if (mom != nullptr && valid) {
        mom[cell] = rho;
        mom[N + cell] = ux;
        mom[2 * N + cell] = uy;
        mom[3 * N + cell] = uz;
        if (THERMAL) {
            // temperature and heat flux sum g c (lbm.cpp:778-792)
            mom[4 * N + cell] = Tc;
            float qx = 0.0f, qy = 0.0f, qz = 0.0f;
#pragma unroll
            for (int l = 1; l < QT; l++) {
                qx += cx(l) * g[l];
                qy += cy(l) * g[l];
                qz += cz(l) * g[l];
            }
            mom[5 * N + cell] = qx;
            mom[6 * N + cell] = qy;
            mom[7 * N + cell] = qz;
        }
    }
    if (export_only || !valid || frozen) return false;

    if (check_band && P.band_on) {
        const int bx = x - ds->band_o[0], by = y - ds->band_o[1], bz = z - ds->band_o[2];
        if ((unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz) {
            const long long nb = P.nb;
            const long long b = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            band[b] = drho;
            band[nb + b] = ux;
            band[2 * nb + b] = uy;
            band[3 * nb + b] = uz;
            band[4 * nb + b] = Fx;
            band[5 * nb + b] = Fy;
            band[6 * nb + b] = Fz;
            band[7 * nb + b] = 0.0f;
            band[8 * nb + b] = 0.0f;
            band[9 * nb + b] = 0.0f;
            band[10 * nb + b] = Tc;
            band[11 * nb + b] = 0.0f;
#pragma unroll
            for (int k = 0; k < 4; k++) P.bandq[k * nb + b] = 0;
            return true;
        }
    }
    collide_flow<float, FORCED>(f, drho, ux, uy, uz, Fx, Fy, Fz, P.omega);
    if (THERMAL) collide_heat<float, false>(g, Tc, ux, uy, uz, 0.0f, P.omega_t);
    return true;
}

// update_cell followed by the stores to B (and GB).
template <class T, bool THERMAL, bool FORCED>
__device__ __forceinline__ void finish_cell(float f[Q], float g[QT], int x, int y, int z, long long cell, bool valid,
                                            int gather, int export_only, T *__restrict__ B, T *__restrict__ GB,
                                            const StepParams &P, DevState *__restrict__ ds, float *__restrict__ mom,
                                            float *__restrict__ band, bool check_band = true, bool frozen = false) {
    if (!update_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, gather, export_only, P, ds, mom, band,
                                         check_band, frozen))
        return;
    if (P.idx32) {
        const unsigned c = (unsigned)cell;
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(B + (c + P.sofs32[l]), f[l]);
    } else {
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
    }
    if (THERMAL) {
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
    }
}

// Collision of band cell b after the IBM forcing iterations: rho and the
// unforced velocity from the step kernel, the accumulated IBM force Ft
// (band[7..9]) and heat source (band[11]).  u = u_unf + Ft / (2 rho) and
// F = Fb + sign Ft (sign = -1 reproduces lbm.cpp:1347-1352);
// T = T_unf + Qt / 2.
template <class T, bool THERMAL>
__device__ __forceinline__ void band_collide_cell(T *__restrict__ B, T *__restrict__ GB, const StepParams &P,
                                                  const DevState *__restrict__ ds, float *__restrict__ band,
                                                  float fsign, long long b) {
    const int bx = (int)(b % P.bsx);
    const int by = (int)((b / P.bsx) % P.bsy);
    const int bz = (int)(b / ((long long)P.bsx * P.bsy));
    const int x = bx + ds->band_o[0], y = by + ds->band_o[1], z = bz + ds->band_o[2];
    if (x < 0 || y < 0 || z < 0 || x >= P.nx || y >= P.ny || z >= P.nz) return;
    const long long nb = P.nb;
    const long long cell = x + (long long)P.nx * (y + (long long)P.ny * z);
    float f[Q];
#pragma unroll
    for (int l = 0; l < Q; l++) f[l] = St<T>::ld(B + l * P.S + cell);
    const float drho = band[b];
    const float rho = 1.0f + drho;
    const float ftx = from_fx(P.bandq[b]), fty = from_fx(P.bandq[nb + b]), ftz = from_fx(P.bandq[2 * nb + b]);
    // the step's IBM force as FP32, for the VTK force density and the
    // free body's internal-fluid momentum
    band[7 * nb + b] = ftx;
    band[8 * nb + b] = fty;
    band[9 * nb + b] = ftz;
    const float ux = band[nb + b] + 0.5f * ftx / rho;
    const float uy = band[2 * nb + b] + 0.5f * fty / rho;
    const float uz = band[3 * nb + b] + 0.5f * ftz / rho;
    const float Fx = band[4 * nb + b] + fsign * ftx;
    const float Fy = band[5 * nb + b] + fsign * fty;
    const float Fz = band[6 * nb + b] + fsign * ftz;
    collide_flow(f, drho, ux, uy, uz, Fx, Fy, Fz, true, P.omega);
#pragma unroll
    for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
    if (THERMAL) {
        float g[QT];
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = St<T>::ld(GB + l * P.S + cell);
        const float Qt = from_fx(P.bandq[3 * nb + b]);
        band[11 * nb + b] = Qt;
        const float Tc = band[10 * nb + b] + 0.5f * Qt;
        collide_heat<float, true>(g, Tc, ux, uy, uz, Qt, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
    }
}

}  // namespace lbmk
