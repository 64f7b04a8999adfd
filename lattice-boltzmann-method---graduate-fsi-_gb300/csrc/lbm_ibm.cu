// lbm_ibm.cu -- immersed-boundary kernels (marker-parallel, one warp per
// marker) and the FP64 force reduction / rigid-body update.
//
// The implicit multi-direct forcing of IBLBM (lbm.cpp:1259-1390) is run on
// the band of cells around the body:
//   k_ibm_interp(first=1): U_m = sum u delta, rho_m = sum rho delta (unforced
//                          moments written by k_step), F_m = 2 rho_m (U_des - U_m)
//   k_ibm_spread:          Ft(x) += F_m ds_m delta(x - X_m)
//   k_ibm_interp(first=0): U_m from u = u_unf + Ft / (2 rho); next F_m
//   ... m_max spreads in total ...
//   k_ibm_finish:          FP64 sums of -F_m ds (drag/lift), torque and heat
//                          in a fixed order; Newton-Euler update when free
//                          (Kempe & Froehlich internal-fluid treatment).
// Each marker's stencil is the 4x4x4 node block with |r| < 2, on which the
// 4-point Peskin delta (lbm.cpp:1095-1102) is non-zero; node (a,b,c) of the
// block is handled by lane a + 4b + 16c (mod 32), two nodes per lane, and the
// warp reduces with shuffles in a fixed order.
#include "lbm_collide.cuh"
#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbmk {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Interpolation at marker m (one warp) and the marker force of the next
// spreading: U_m = sum u delta with u = u_unf + Ft / (2 rho), rho_m on the
// first pass, F_m = 2 rho_m (U_des - U_m); the FP64 accumulators collect
// -F_m ds (the reference's Drag/Lift sums, lbm.cpp:1322-1323) and Q_m ds.
__device__ __forceinline__ void interp_marker(int m, int lane, const StepParams &P, const MarkerDev &mk,
                                              DevState *__restrict__ ds, const float *__restrict__ band, int first,
                                              int thermal) {
    const int n = mk.n;
    const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
    const double flx = floor(X), fly = floor(Y), flz = floor(Z);
    const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
    // stencil node a: reference node i = floor(X) - 1 + a, device cell i - 1
    const int bx0 = (int)flx - 2 - ds->band_o[0];
    const int by0 = (int)fly - 2 - ds->band_o[1];
    const int bz0 = (int)flz - 2 - ds->band_o[2];
    const long long nb = P.nb;
    float su = 0.f, sv = 0.f, sw = 0.f, sr = 0.f, sT = 0.f;
    bool edge = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        const float wgt = peskin((float)(a - 1) - fx) * peskin((float)(b - 1) - fy) * peskin((float)(c - 1) - fz);
        const int bx = bx0 + a, by = by0 + b, bz = bz0 + c;
        if ((unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            const float rho = 1.0f + band[q];
            const float hr = 0.5f / rho;
            su += wgt * (band[nb + q] + hr * band[7 * nb + q]);
            sv += wgt * (band[2 * nb + q] + hr * band[8 * nb + q]);
            sw += wgt * (band[3 * nb + q] + hr * band[9 * nb + q]);
            if (first) sr += wgt * rho;
            if (thermal) sT += wgt * (band[10 * nb + q] + 0.5f * band[11 * nb + q]);
        } else if (wgt != 0.0f) {
            edge = true;
        }
    }
    su = warp_sum(su);
    sv = warp_sum(sv);
    sw = warp_sum(sw);
    if (first) sr = warp_sum(sr);
    if (thermal) sT = warp_sum(sT);
    const bool any_edge = __any_sync(0xffffffffu, edge);
    if (lane == 0) {
        if (any_edge) atomicOr(&ds->status, ST_BAND_EDGE);
        if (first) mk.rho[m] = sr;
        const float rm = first ? sr : mk.rho[m];
        const float Fx = 2.0f * rm * (mk.udes[m] - su);
        const float Fy = 2.0f * rm * (mk.udes[n + m] - sv);
        const float Fz = 2.0f * rm * (mk.udes[2 * n + m] - sw);
        mk.force[m] = Fx;
        mk.force[n + m] = Fy;
        mk.force[2 * n + m] = Fz;
        const double dsv = mk.ds[m];
        mk.acc[m] += -(double)Fx * dsv;
        mk.acc[n + m] += -(double)Fy * dsv;
        mk.acc[2 * n + m] += -(double)Fz * dsv;
        if (thermal) {
            const float Qm = 2.0f * (mk.tdes - sT);
            mk.force[3 * n + m] = Qm;
            mk.acc[3 * n + m] += (double)Qm * dsv;
        }
        if (!isfinite(Fx) || !isfinite(Fy) || !isfinite(Fz)) atomicOr(&ds->status, ST_NONFINITE_FORCE);
    }
}

// Spreading of marker m (one warp): Ft(x) += F_m ds_m delta(x - X_m)
// (lbm.cpp:1331-1360), float atomics into the band.
__device__ __forceinline__ void spread_marker(int m, int lane, const StepParams &P, const MarkerDev &mk,
                                              const DevState *__restrict__ ds, float *__restrict__ band,
                                              int thermal) {
    const int n = mk.n;
    const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
    const double flx = floor(X), fly = floor(Y), flz = floor(Z);
    const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
    const int bx0 = (int)flx - 2 - ds->band_o[0];
    const int by0 = (int)fly - 2 - ds->band_o[1];
    const int bz0 = (int)flz - 2 - ds->band_o[2];
    const long long nb = P.nb;
    const float dsv = (float)mk.ds[m];
    const float Fx = mk.force[m] * dsv, Fy = mk.force[n + m] * dsv, Fz = mk.force[2 * n + m] * dsv;
    const float Qm = thermal ? mk.force[3 * n + m] * dsv : 0.0f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        const float wgt = peskin((float)(a - 1) - fx) * peskin((float)(b - 1) - fy) * peskin((float)(c - 1) - fz);
        const int bx = bx0 + a, by = by0 + b, bz = bz0 + c;
        if (wgt != 0.0f && (unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy &&
            (unsigned)bz < (unsigned)P.bsz) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            atomicAdd(&band[7 * nb + q], Fx * wgt);
            atomicAdd(&band[8 * nb + q], Fy * wgt);
            atomicAdd(&band[9 * nb + q], Fz * wgt);
            if (thermal) atomicAdd(&band[11 * nb + q], Qm * wgt);
        }
    }
}

__global__ void __launch_bounds__(128) k_ibm_interp(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    DevState *__restrict__ ds, const float *__restrict__ band,
                                                    int first, int thermal) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (m >= mk.n) return;  // whole warp leaves together
    interp_marker(m, threadIdx.x & 31, P, mk, ds, band, first, thermal);
}

__global__ void __launch_bounds__(128) k_ibm_spread(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    const DevState *__restrict__ ds, float *__restrict__ band,
                                                    int thermal) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (m >= mk.n) return;
    spread_marker(m, threadIdx.x & 31, P, mk, ds, band, thermal);
}

// One block.  Deterministic FP64 reductions: each thread sums a strided set
// in index order, then a fixed shared-memory tree.
__device__ __forceinline__ void block_tree(double (*red)[256], int nq, int t) {
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < nq; k++) red[k][t] += red[k][t + w];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_ibm_finish(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    DevState *__restrict__ ds, BodyParams bp,
                                                    const float *__restrict__ band, double *__restrict__ hist,
                                                    long long hist_cap) {
    __shared__ double red[7][256];
    __shared__ double sh_dxc[3], sh_om[3], sh_v[3], sh_xc[3], sh_f[7];
    const int t = threadIdx.x;
    const int n = mk.n;
    const double xc0 = ds->body_xc[0], xc1 = ds->body_xc[1], xc2 = ds->body_xc[2];
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int m = t; m < n; m += 256) {
        const double fx = mk.acc[m], fy = mk.acc[n + m], fz = mk.acc[2 * n + m], hq = mk.acc[3 * n + m];
        const double rx = mk.pos[m] - xc0, ry = mk.pos[n + m] - xc1, rz = mk.pos[2 * n + m] - xc2;
        s[0] += fx;
        s[1] += fy;
        s[2] += fz;
        s[3] += ry * fz - rz * fy;
        s[4] += rz * fx - rx * fz;
        s[5] += rx * fy - ry * fx;
        s[6] += hq;
        mk.acc[m] = 0.0;
        mk.acc[n + m] = 0.0;
        mk.acc[2 * n + m] = 0.0;
        mk.acc[3 * n + m] = 0.0;
    }
#pragma unroll
    for (int k = 0; k < 7; k++) red[k][t] = s[k];
    block_tree(red, 7, t);
    if (t == 0) {
        const long long step = ds->step;
        double *h = hist + (step % hist_cap) * 8;
        for (int k = 0; k < 7; k++) {
            h[k] = red[k][0];
            sh_f[k] = red[k][0];
        }
        h[7] = (double)step;
        ds->step = step + 1;
    }
    if (!bp.free_body) return;
    // fluid momentum and angular momentum inside the body after the forced
    // collision, u_unf + F_b / (2 rho) + Ft / rho, volume fraction
    // clamp(R + 1/2 - |x - xc|, 0, 1) (Kempe & Froehlich 2012)
    __syncthreads();
    double q[6] = {0, 0, 0, 0, 0, 0};
    const long long nb = P.nb;
    for (long long b = t; b < nb; b += 256) {
        const int bx = (int)(b % P.bsx), by = (int)((b / P.bsx) % P.bsy), bz = (int)(b / ((long long)P.bsx * P.bsy));
        const int x = bx + ds->band_o[0], y = by + ds->band_o[1], z = bz + ds->band_o[2];
        if (x >= P.nx || y >= P.ny || z >= P.nz) continue;
        const double rx = (x + 1) - xc0, ry = (y + 1) - xc1, rz = (z + 1) - xc2;
        double a = bp.radius + 0.5 - sqrt(rx * rx + ry * ry + rz * rz);
        if (a <= 0.0) continue;
        if (a > 1.0) a = 1.0;
        const double rho = 1.0 + (double)band[b];
        const double ux = (double)band[nb + b] + 0.5 * band[4 * nb + b] / rho + band[7 * nb + b] / rho;
        const double uy = (double)band[2 * nb + b] + 0.5 * band[5 * nb + b] / rho + band[8 * nb + b] / rho;
        const double uz = (double)band[3 * nb + b] + 0.5 * band[6 * nb + b] / rho + band[9 * nb + b] / rho;
        q[0] += a * ux;
        q[1] += a * uy;
        q[2] += a * uz;
        q[3] += a * (ry * uz - rz * uy);
        q[4] += a * (rz * ux - rx * uz);
        q[5] += a * (rx * uy - ry * ux);
    }
#pragma unroll
    for (int k = 0; k < 6; k++) red[k][t] = q[k];
    block_tree(red, 6, t);
    if (t == 0) {
        if (!ds->have_prev) {
            for (int k = 0; k < 6; k++) ds->internal_prev[k] = red[k][0];
            ds->have_prev = 1;
        }
        // Newton-Euler, dt = 1: rho_s V dV/dt = F_h + dI/dt + (rho_s - rho_f) V g
        for (int a = 0; a < 3; a++) {
            const double dI = red[a][0] - ds->internal_prev[a];
            const double dL = red[3 + a][0] - ds->internal_prev[3 + a];
            const double vn =
                ((bp.dof >> a) & 1) ? ds->body_v[a] + (sh_f[a] + dI) / bp.mass + bp.gacc[a] : ds->body_v[a];
            const double om =
                ((bp.dof >> (3 + a)) & 1) ? ds->body_om[a] + (sh_f[3 + a] + dL) / bp.inertia : ds->body_om[a];
            const double d = 0.5 * (ds->body_v[a] + vn);
            sh_dxc[a] = d;
            sh_v[a] = vn;
            sh_om[a] = om;
            sh_xc[a] = ds->body_xc[a] + d;
            ds->body_dxc[a] = d;
            ds->body_v[a] = vn;
            ds->body_om[a] = om;
            ds->body_xc[a] = sh_xc[a];
        }
        for (int k = 0; k < 6; k++) ds->internal_prev[k] = red[k][0];
        const int ns[3] = {P.nx, P.ny, P.nz};
        const int bs[3] = {P.bsx, P.bsy, P.bsz};
        for (int a = 0; a < 3; a++) {
            int o = (int)floor(sh_xc[a] - bp.radius) - 2;
            o = max(0, min(o, ns[a] - bs[a]));
            ds->band_o[a] = o;
        }
    }
    __syncthreads();
    const double R = bp.radius;
    for (int m = t; m < n; m += 256) {
        const double r0 = mk.pos[m] - (sh_xc[0] - sh_dxc[0]);
        const double r1 = mk.pos[n + m] - (sh_xc[1] - sh_dxc[1]);
        const double r2 = mk.pos[2 * n + m] - (sh_xc[2] - sh_dxc[2]);
        double q0 = r0 + (sh_om[1] * r2 - sh_om[2] * r1);
        double q1 = r1 + (sh_om[2] * r0 - sh_om[0] * r2);
        double q2 = r2 + (sh_om[0] * r1 - sh_om[1] * r0);
        const double sc = R / sqrt(q0 * q0 + q1 * q1 + q2 * q2);
        q0 *= sc;
        q1 *= sc;
        q2 *= sc;
        mk.pos[m] = sh_xc[0] + q0;
        mk.pos[n + m] = sh_xc[1] + q1;
        mk.pos[2 * n + m] = sh_xc[2] + q2;
        mk.udes[m] = (float)(sh_v[0] + (sh_om[1] * q2 - sh_om[2] * q1));
        mk.udes[n + m] = (float)(sh_v[1] + (sh_om[2] * q0 - sh_om[0] * q2));
        mk.udes[2 * n + m] = (float)(sh_v[2] + (sh_om[0] * q1 - sh_om[1] * q0));
    }
}

// ---------------------------------------------------------------------------
// Assembled IBM phase (rigid bodies whose marker pattern only translates).
// The implicit iteration of lbm.cpp:1311-1388 is linear in the accumulated
// marker forces: with u(x) = u_unf(x) + Ft(x) / (2 rho(x)) and
// Ft = sum_n Ftot_n ds_n delta_n,
//     U_m = U0_m + sum_n A_mn ds_n Ftot_n,
//     A_mn = sum_x delta_m(x) delta_n(x) / (2 rho(x)),
// so the m_max passes run in marker space once A is assembled:
//   k_ibm_prep      (warp per marker) U0_m, rho_m (and T0_m) by
//                   interpolation, and the row of A (and of the heat
//                   coupling, delta delta / 2) over the marker's neighbours;
//   k_ibm_iterate   (one CTA) the m_max passes, F_m = 2 rho_m (U_des - U_m),
//                   Ftot_m += F_m, FP64 -F_m ds sums; for a fixed body also
//                   the force/torque/heat totals and the history entry;
//   k_ibm_gather_collide (band cell) Ft(x) = sum over the markers covering
//                   x of Ftot_m ds_m delta_m(x), then the band collision.
// Same arithmetic as the kernel chain up to the order of the sums.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_ibm_prep(const __grid_constant__ StepParams P, MarkerDev mk,
                                                  DevState *__restrict__ ds, const float *__restrict__ band,
                                                  const int *__restrict__ pair_ptr, const int *__restrict__ pair_idx,
                                                  float *__restrict__ pairA, float *__restrict__ pairB, int heat) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= mk.n) return;
    const int n = mk.n;
    const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
    const double flx = floor(X), fly = floor(Y), flz = floor(Z);
    const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
    const int bx0 = (int)flx - 2 - ds->band_o[0];
    const int by0 = (int)fly - 2 - ds->band_o[1];
    const int bz0 = (int)flz - 2 - ds->band_o[2];
    const long long nb = P.nb;
    float wgt[2], hr[2];
    int nodei[2][3];
    bool inb[2];
    float su = 0.f, sv = 0.f, sw = 0.f, sr = 0.f, sT = 0.f;
    bool edge = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        wgt[h] = peskin((float)(a - 1) - fx) * peskin((float)(b - 1) - fy) * peskin((float)(c - 1) - fz);
        nodei[h][0] = (int)flx - 1 + a;  // reference node coordinates
        nodei[h][1] = (int)fly - 1 + b;
        nodei[h][2] = (int)flz - 1 + c;
        const int bx = bx0 + a, by = by0 + b, bz = bz0 + c;
        inb[h] = (unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz;
        hr[h] = 0.0f;
        if (inb[h]) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            const float rho = 1.0f + band[q];
            hr[h] = 0.5f / rho;
            su += wgt[h] * band[nb + q];
            sv += wgt[h] * band[2 * nb + q];
            sw += wgt[h] * band[3 * nb + q];
            sr += wgt[h] * rho;
            if (heat) sT += wgt[h] * band[10 * nb + q];
        } else if (wgt[h] != 0.0f) {
            edge = true;
        }
    }
    su = warp_sum(su);
    sv = warp_sum(sv);
    sw = warp_sum(sw);
    sr = warp_sum(sr);
    if (heat) sT = warp_sum(sT);
    if (__any_sync(0xffffffffu, edge) && lane == 0) atomicOr(&ds->status, ST_BAND_EDGE);
    if (lane == 0) {
        mk.u0[m] = su;
        mk.u0[n + m] = sv;
        mk.u0[2 * n + m] = sw;
        mk.rho[m] = sr;
        mk.t0[m] = sT;
    }
    // row m of the coupling matrices
    for (int k = pair_ptr[m]; k < pair_ptr[m + 1]; k++) {
        const int j = pair_idx[k];
        const double Xj = mk.pos[j], Yj = mk.pos[n + j], Zj = mk.pos[2 * n + j];
        float am = 0.f, bm = 0.f;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            if (!inb[h] || wgt[h] == 0.0f) continue;
            const float rx = (float)(nodei[h][0] - Xj), ry = (float)(nodei[h][1] - Yj), rz = (float)(nodei[h][2] - Zj);
            if (fabsf(rx) >= 2.0f || fabsf(ry) >= 2.0f || fabsf(rz) >= 2.0f) continue;
            const float wj = peskin(rx) * peskin(ry) * peskin(rz);
            am += wgt[h] * wj * hr[h];
            bm += wgt[h] * wj * 0.5f;
        }
        am = warp_sum(am);
        if (heat) bm = warp_sum(bm);
        if (lane == 0) {
            pairA[k] = am;
            if (heat) pairB[k] = bm;
        }
    }
}

// One CTA.  Marker state lives in shared memory between the passes.
__global__ void __launch_bounds__(1024) k_ibm_iterate(const __grid_constant__ StepParams P, MarkerDev mk,
                                                      DevState *__restrict__ ds, const int *__restrict__ pair_ptr,
                                                      const int *__restrict__ pair_idx,
                                                      const float *__restrict__ pairA,
                                                      const float *__restrict__ pairB, int m_max, int heat,
                                                      int write_history, double *__restrict__ hist,
                                                      long long hist_cap) {
    extern __shared__ float sm[];  // [4][n] of ds_m Ftot_m (x, y, z) and ds_m Qtot_m
    __shared__ double red[7][32];
    const int n = mk.n;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < 4 * n; i += nt) sm[i] = 0.0f;
    __syncthreads();
    double acc[4][4];  // up to 4 markers per thread x (fx, fy, fz, q)
    for (int r = 0; r < 4; r++)
        for (int q = 0; q < 4; q++) acc[r][q] = 0.0;
    for (int it = 0; it < m_max; it++) {
        float Fn[4][4];
        for (int r = 0; r < 4; r++) {
            const int m = tid + r * nt;
            if (m >= n) break;
            float ux = mk.u0[m], uy = mk.u0[n + m], uz = mk.u0[2 * n + m], T = mk.t0[m];
            for (int k = pair_ptr[m]; k < pair_ptr[m + 1]; k++) {
                const int j = pair_idx[k];
                const float a = pairA[k];
                ux += a * sm[j];
                uy += a * sm[n + j];
                uz += a * sm[2 * n + j];
                if (heat) T += pairB[k] * sm[3 * n + j];
            }
            const float rm = mk.rho[m];
            Fn[r][0] = 2.0f * rm * (mk.udes[m] - ux);
            Fn[r][1] = 2.0f * rm * (mk.udes[n + m] - uy);
            Fn[r][2] = 2.0f * rm * (mk.udes[2 * n + m] - uz);
            Fn[r][3] = heat ? 2.0f * (mk.tdes - T) : 0.0f;
        }
        __syncthreads();  // every read of this pass's Ftot is done
        for (int r = 0; r < 4; r++) {
            const int m = tid + r * nt;
            if (m >= n) break;
            const float dsm = (float)mk.ds[m];
            const double dsd = mk.ds[m];
            for (int q = 0; q < 4; q++) {
                sm[q * n + m] += dsm * Fn[r][q];
                acc[r][q] += (q < 3 ? -(double)Fn[r][q] : (double)Fn[r][q]) * dsd;
            }
            if (!isfinite(Fn[r][0]) || !isfinite(Fn[r][1]) || !isfinite(Fn[r][2]))
                atomicOr(&ds->status, ST_NONFINITE_FORCE);
        }
        __syncthreads();
    }
    // ds_m Ftot_m for the spreading, FP64 accumulators for the finish
    for (int r = 0; r < 4; r++) {
        const int m = tid + r * nt;
        if (m >= n) break;
        for (int q = 0; q < 4; q++) {
            mk.force[q * n + m] = sm[q * n + m];
            mk.acc[q * n + m] = acc[r][q];
        }
    }
    if (!write_history) return;
    // fixed body: totals in a fixed order (thread, then warp tree, then warps)
    const double xc0 = ds->body_xc[0], xc1 = ds->body_xc[1], xc2 = ds->body_xc[2];
    double s7[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int r = 0; r < 4; r++) {
        const int m = tid + r * nt;
        if (m >= n) break;
        const double rx = mk.pos[m] - xc0, ry = mk.pos[n + m] - xc1, rz = mk.pos[2 * n + m] - xc2;
        const double fx = acc[r][0], fy = acc[r][1], fz = acc[r][2];
        s7[0] += fx;
        s7[1] += fy;
        s7[2] += fz;
        s7[3] += ry * fz - rz * fy;
        s7[4] += rz * fx - rx * fz;
        s7[5] += rx * fy - ry * fx;
        s7[6] += acc[r][3];
    }
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int q = 0; q < 7; q++) {
        double v = s7[q];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[q][w] = v;
    }
    __syncthreads();
    if (tid == 0) {
        const long long step = ds->step;
        double *h = hist + (step % hist_cap) * 8;
        for (int q = 0; q < 7; q++) {
            double v = 0.0;
            for (int i = 0; i < (nt >> 5); i++) v += red[q][i];
            h[q] = v;
        }
        h[7] = (double)step;
        ds->step = step + 1;
    }
}

// Band cell: Ft(x) and Qt(x) gathered from the markers that cover it, then
// the band collision (k_band_collide's arithmetic).
template <class T, bool THERMAL>
__global__ void __launch_bounds__(256) k_ibm_gather_collide(T *__restrict__ B, T *__restrict__ GB,
                                                            const __grid_constant__ StepParams P, MarkerDev mk,
                                                            const DevState *__restrict__ ds, float *__restrict__ band,
                                                            const int *__restrict__ node_ptr,
                                                            const int *__restrict__ node_mk, float fsign, int heat) {
    const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (b >= P.nb) return;
    const int bx = (int)(b % P.bsx), by = (int)((b / P.bsx) % P.bsy), bz = (int)(b / ((long long)P.bsx * P.bsy));
    const int x = bx + ds->band_o[0], y = by + ds->band_o[1], z = bz + ds->band_o[2];
    const long long nb = P.nb;
    const int n = mk.n;
    float ftx = 0.f, fty = 0.f, ftz = 0.f, qt = 0.f;
    for (int k = node_ptr[b]; k < node_ptr[b + 1]; k++) {
        const int m = node_mk[k];
        const float rx = (float)((x + 1) - mk.pos[m]), ry = (float)((y + 1) - mk.pos[n + m]),
                    rz = (float)((z + 1) - mk.pos[2 * n + m]);
        const float w = peskin(rx) * peskin(ry) * peskin(rz);
        ftx += mk.force[m] * w;
        fty += mk.force[n + m] * w;
        ftz += mk.force[2 * n + m] * w;
        if (heat) qt += mk.force[3 * n + m] * w;
    }
    band[7 * nb + b] = ftx;
    band[8 * nb + b] = fty;
    band[9 * nb + b] = ftz;
    band[11 * nb + b] = qt;
    if (x < 0 || y < 0 || z < 0 || x >= P.nx || y >= P.ny || z >= P.nz) return;
    const long long cell = x + (long long)P.nx * (y + (long long)P.ny * z);
    float f[Q];
#pragma unroll
    for (int l = 0; l < Q; l++) f[l] = St<T>::ld(B + l * P.S + cell);
    const float drho = band[b];
    const float rho = 1.0f + drho;
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
        const float Tc = band[10 * nb + b] + 0.5f * qt;
        collide_heat(g, Tc, ux, uy, uz, qt, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
    }
}

// Moving body: spread the accumulated ds_m Ftot_m with float atomics.
__global__ void __launch_bounds__(128) k_ibm_spread_total(const __grid_constant__ StepParams P, MarkerDev mk,
                                                          const DevState *__restrict__ ds, float *__restrict__ band,
                                                          int heat) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= mk.n) return;
    const int n = mk.n;
    const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
    const double flx = floor(X), fly = floor(Y), flz = floor(Z);
    const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
    const int bx0 = (int)flx - 2 - ds->band_o[0];
    const int by0 = (int)fly - 2 - ds->band_o[1];
    const int bz0 = (int)flz - 2 - ds->band_o[2];
    const long long nb = P.nb;
    const float Fx = mk.force[m], Fy = mk.force[n + m], Fz = mk.force[2 * n + m], Qm = mk.force[3 * n + m];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        const float wgt = peskin((float)(a - 1) - fx) * peskin((float)(b - 1) - fy) * peskin((float)(c - 1) - fz);
        const int bx = bx0 + a, by = by0 + b, bz = bz0 + c;
        if (wgt != 0.0f && (unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy &&
            (unsigned)bz < (unsigned)P.bsz) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            atomicAdd(&band[7 * nb + q], Fx * wgt);
            atomicAdd(&band[8 * nb + q], Fy * wgt);
            atomicAdd(&band[9 * nb + q], Fz * wgt);
            if (heat) atomicAdd(&band[11 * nb + q], Qm * wgt);
        }
    }
}

cudaError_t lbmk_iterate_smem(int n_markers) {
    return cudaFuncSetAttribute(k_ibm_iterate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)((size_t)4 * n_markers * sizeof(float)));
}

cudaError_t launch_ibm_assembled(int storage, bool lattice_thermal, const IbmArgs &a, const AsmPlan &ap, void *B,
                                 void *GB, float fsign, int m_max, double *hist, long long hist_cap,
                                 const BodyParams &bp, const LaunchArgs &la) {
    const long long warps_blocks = ((long long)a.mk.n * 32 + 127) / 128;
    k_ibm_prep<<<(unsigned)warps_blocks, 128, 0, a.stream>>>(*a.P, a.mk, a.ds, a.band, ap.pair_ptr, ap.pair_idx,
                                                            ap.pairA, ap.pairB, a.thermal);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const size_t smem = (size_t)4 * a.mk.n * sizeof(float);
    k_ibm_iterate<<<1, 1024, smem, a.stream>>>(*a.P, a.mk, a.ds, ap.pair_ptr, ap.pair_idx, ap.pairA, ap.pairB, m_max,
                                               a.thermal, bp.free_body ? 0 : 1, hist, hist_cap);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const long long nb = a.P->nb;
    const unsigned bblocks = (unsigned)((nb + 255) / 256);
    if (!bp.free_body && ap.node_ptr) {
#define GC_LAUNCH(TT, TH)                                                                                      \
    k_ibm_gather_collide<TT, TH><<<bblocks, 256, 0, a.stream>>>((TT *)B, (TT *)GB, *a.P, a.mk, a.ds, a.band,  \
                                                               ap.node_ptr, ap.node_mk, fsign, a.thermal)
        switch (storage) {
        case 0: if (lattice_thermal) GC_LAUNCH(float, true); else GC_LAUNCH(float, false); break;
        case 1: if (lattice_thermal) GC_LAUNCH(__half, true); else GC_LAUNCH(__half, false); break;
        case 2: if (lattice_thermal) GC_LAUNCH(__nv_bfloat16, true); else GC_LAUNCH(__nv_bfloat16, false); break;
        }
#undef GC_LAUNCH
        return cudaGetLastError();
    }
    k_ibm_spread_total<<<(unsigned)warps_blocks, 128, 0, a.stream>>>(*a.P, a.mk, a.ds, a.band, a.thermal);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = launch_band_collide(storage, la, fsign)) != cudaSuccess) return e;
    return launch_ibm_finish(a, bp, hist, hist_cap);
}

cudaError_t launch_ibm_interp(const IbmArgs &a, int first) {
    const int threads = 128;
    const long long blocks = ((long long)a.mk.n * 32 + threads - 1) / threads;
    k_ibm_interp<<<(unsigned)blocks, threads, 0, a.stream>>>(*a.P, a.mk, a.ds, a.band, first, a.thermal);
    return cudaGetLastError();
}

cudaError_t launch_ibm_spread(const IbmArgs &a) {
    const int threads = 128;
    const long long blocks = ((long long)a.mk.n * 32 + threads - 1) / threads;
    k_ibm_spread<<<(unsigned)blocks, threads, 0, a.stream>>>(*a.P, a.mk, a.ds, a.band, a.thermal);
    return cudaGetLastError();
}

cudaError_t launch_ibm_finish(const IbmArgs &a, const BodyParams &bp, double *hist, long long hist_cap) {
    k_ibm_finish<<<1, 256, 0, a.stream>>>(*a.P, a.mk, a.ds, bp, a.band, hist, hist_cap);
    return cudaGetLastError();
}

}  // namespace lbmk
