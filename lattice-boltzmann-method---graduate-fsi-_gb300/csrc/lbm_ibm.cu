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
#include <cooperative_groups.h>

#include "lbm_collide.cuh"
#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace cg = cooperative_groups;

namespace lbmk {

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(128) k_ibm_interp(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    DevState *__restrict__ ds, const float *__restrict__ band,
                                                    int first, int thermal) {
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (m >= mk.n) return;  // whole warp leaves together
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

__global__ void __launch_bounds__(128) k_ibm_spread(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    const DevState *__restrict__ ds, float *__restrict__ band,
                                                    int thermal) {
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
// Fused IBM step: one thread-block cluster runs the whole forcing phase of a
// time step -- m_max interpolate/spread iterations, the band collision, the
// FP64 force/torque/heat sums and the rigid-body update -- in one launch.
// The band is split into z slabs, one per CTA, held in shared memory; a
// marker's 4x4x4 stencil may straddle slabs, so interpolation reads and
// spreading atomics go to the owning CTA's shared memory through the cluster
// (distributed shared memory).  Phases are separated by hardware cluster
// barriers.  Marker m belongs to CTA m % CL.
//   smem: [NF][slab cells] floats: rho, u_unf(3), Ft(3), (T_unf, Qt)
//         then per owned marker: F(4) + rho_m floats, acc(4) doubles,
//         then 16 doubles of partial sums.
// ---------------------------------------------------------------------------
template <class T, bool THERMAL>
__global__ void __launch_bounds__(512, 1) k_ibm_fused(T *__restrict__ B, T *__restrict__ GB,
                                                       const __grid_constant__ StepParams P, MarkerDev mk,
                                                       DevState *__restrict__ ds, float *__restrict__ band,
                                                       BodyParams bp, double *__restrict__ hist, long long hist_cap,
                                                       int m_max, float fsign, int slab, int nloc_max, int heat) {
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int NF = THERMAL ? 9 : 7;
    const int CL = (int)cluster.num_blocks();
    const int r = (int)cluster.block_rank();
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    const int bsx = P.bsx, bsy = P.bsy, bsz = P.bsz;
    const long long nb = P.nb;
    const int plane = bsx * bsy;
    const int slab_cells = slab * plane;
    const int z_lo = r * slab;
    const int z_hi = min(bsz, z_lo + slab);
    const int my_cells = max(0, z_hi - z_lo) * plane;
    float *fld = reinterpret_cast<float *>(smem);                           // [NF][slab_cells]
    float *mF = fld + (size_t)NF * slab_cells;                              // [4][nloc_max]
    float *mR = mF + 4 * nloc_max;                                          // [nloc_max]
    double *mA = reinterpret_cast<double *>(
        smem + ((((size_t)NF * slab_cells + 5 * (size_t)nloc_max) * sizeof(float) + 15) / 16) * 16);  // [4][nloc_max]
    double *part = mA + 4 * nloc_max;                                       // [16]
    const int o0 = ds->band_o[0], o1 = ds->band_o[1], o2 = ds->band_o[2];
    const int n = mk.n;
    const int nloc = n > r ? (n - r + CL - 1) / CL : 0;

    // load this CTA's slab of the band written by k_step
    for (int c = tid; c < my_cells; c += nthr) {
        const long long b = (long long)z_lo * plane + c;
        fld[c] = 1.0f + band[b];
        fld[slab_cells + c] = band[nb + b];
        fld[2 * slab_cells + c] = band[2 * nb + b];
        fld[3 * slab_cells + c] = band[3 * nb + b];
        fld[4 * slab_cells + c] = 0.0f;
        fld[5 * slab_cells + c] = 0.0f;
        fld[6 * slab_cells + c] = 0.0f;
        if (THERMAL) {
            fld[7 * slab_cells + c] = band[10 * nb + b];
            fld[8 * slab_cells + c] = 0.0f;
        }
    }
    for (int k = tid; k < 4 * nloc_max; k += nthr) mA[k] = 0.0;
    cluster.sync();

    bool edge = false;
    for (int it = 1; it <= m_max; it++) {
        // interpolation and marker force (lbm.cpp:1288-1324)
        for (int k = warp; k < nloc; k += nwarps) {
            const int m = r + CL * k;
            const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
            const double flx = floor(X), fly = floor(Y), flz = floor(Z);
            const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
            const int bx0 = (int)flx - 2 - o0, by0 = (int)fly - 2 - o1, bz0 = (int)flz - 2 - o2;
            float su = 0.f, sv = 0.f, sw = 0.f, sr = 0.f, sT = 0.f;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int s = lane + 32 * h;
                const int a = s & 3, bb = (s >> 2) & 3, cc = s >> 4;
                const float wgt = peskin((float)(a - 1) - fx) * peskin((float)(bb - 1) - fy) * peskin((float)(cc - 1) - fz);
                const int bx = bx0 + a, by = by0 + bb, bz = bz0 + cc;
                if ((unsigned)bx < (unsigned)bsx && (unsigned)by < (unsigned)bsy && (unsigned)bz < (unsigned)bsz) {
                    const int q = bz / slab;
                    const int li = (bz - q * slab) * plane + by * bsx + bx;
                    const float *rf = cluster.map_shared_rank(fld, q);
                    const float rho = rf[li];
                    const float hr = 0.5f / rho;
                    su += wgt * (rf[slab_cells + li] + hr * rf[4 * slab_cells + li]);
                    sv += wgt * (rf[2 * slab_cells + li] + hr * rf[5 * slab_cells + li]);
                    sw += wgt * (rf[3 * slab_cells + li] + hr * rf[6 * slab_cells + li]);
                    if (it == 1) sr += wgt * rho;
                    if (THERMAL && heat) sT += wgt * (rf[7 * slab_cells + li] + 0.5f * rf[8 * slab_cells + li]);
                } else if (wgt != 0.0f) {
                    edge = true;
                }
            }
            su = warp_sum(su);
            sv = warp_sum(sv);
            sw = warp_sum(sw);
            if (it == 1) sr = warp_sum(sr);
            if (THERMAL && heat) sT = warp_sum(sT);
            if (lane == 0) {
                if (it == 1) mR[k] = sr;
                const float rm = mR[k];
                const float Fx = 2.0f * rm * (mk.udes[m] - su);
                const float Fy = 2.0f * rm * (mk.udes[n + m] - sv);
                const float Fz = 2.0f * rm * (mk.udes[2 * n + m] - sw);
                mF[k] = Fx;
                mF[nloc_max + k] = Fy;
                mF[2 * nloc_max + k] = Fz;
                const double dsv = mk.ds[m];
                mA[k] += -(double)Fx * dsv;
                mA[nloc_max + k] += -(double)Fy * dsv;
                mA[2 * nloc_max + k] += -(double)Fz * dsv;
                if (THERMAL && heat) {
                    const float Qm = 2.0f * (mk.tdes - sT);
                    mF[3 * nloc_max + k] = Qm;
                    mA[3 * nloc_max + k] += (double)Qm * dsv;
                }
                if (!isfinite(Fx) || !isfinite(Fy) || !isfinite(Fz)) atomicOr(&ds->status, ST_NONFINITE_FORCE);
            }
        }
        cluster.sync();
        // spreading (lbm.cpp:1331-1360) into the owners' Ft
        for (int k = warp; k < nloc; k += nwarps) {
            const int m = r + CL * k;
            const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
            const double flx = floor(X), fly = floor(Y), flz = floor(Z);
            const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
            const int bx0 = (int)flx - 2 - o0, by0 = (int)fly - 2 - o1, bz0 = (int)flz - 2 - o2;
            const float dsv = (float)mk.ds[m];
            const float Fx = mF[k] * dsv, Fy = mF[nloc_max + k] * dsv, Fz = mF[2 * nloc_max + k] * dsv;
            const float Qm = (THERMAL && heat) ? mF[3 * nloc_max + k] * dsv : 0.0f;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int s = lane + 32 * h;
                const int a = s & 3, bb = (s >> 2) & 3, cc = s >> 4;
                const float wgt = peskin((float)(a - 1) - fx) * peskin((float)(bb - 1) - fy) * peskin((float)(cc - 1) - fz);
                const int bx = bx0 + a, by = by0 + bb, bz = bz0 + cc;
                if (wgt != 0.0f && (unsigned)bx < (unsigned)bsx && (unsigned)by < (unsigned)bsy &&
                    (unsigned)bz < (unsigned)bsz) {
                    const int q = bz / slab;
                    const int li = (bz - q * slab) * plane + by * bsx + bx;
                    float *rf = cluster.map_shared_rank(fld, q);
                    atomicAdd(&rf[4 * slab_cells + li], Fx * wgt);
                    atomicAdd(&rf[5 * slab_cells + li], Fy * wgt);
                    atomicAdd(&rf[6 * slab_cells + li], Fz * wgt);
                    if (THERMAL && heat) atomicAdd(&rf[8 * slab_cells + li], Qm * wgt);
                }
            }
        }
        cluster.sync();
    }
    if (__any_sync(0xffffffffu, edge) && lane == 0) atomicOr(&ds->status, ST_BAND_EDGE);

    // band collision (k_band_collide's arithmetic) on this CTA's slab
    for (int c = tid; c < my_cells; c += nthr) {
        const int bz = z_lo + c / plane, rem = c % plane, by = rem / bsx, bx = rem % bsx;
        const int x = bx + o0, y = by + o1, z = bz + o2;
        if (x >= P.nx || y >= P.ny || z >= P.nz) continue;
        const long long b = (long long)bz * plane + by * bsx + bx;
        const long long cell = x + (long long)P.nx * (y + (long long)P.ny * z);
        float f[Q];
#pragma unroll
        for (int l = 0; l < Q; l++) f[l] = St<T>::ld(B + l * P.S + cell);
        const float rho = fld[c];
        const float ftx = fld[4 * slab_cells + c], fty = fld[5 * slab_cells + c], ftz = fld[6 * slab_cells + c];
        const float ux = fld[slab_cells + c] + 0.5f * ftx / rho;
        const float uy = fld[2 * slab_cells + c] + 0.5f * fty / rho;
        const float uz = fld[3 * slab_cells + c] + 0.5f * ftz / rho;
        const float Fx = band[4 * nb + b] + fsign * ftx;
        const float Fy = band[5 * nb + b] + fsign * fty;
        const float Fz = band[6 * nb + b] + fsign * ftz;
        collide_flow(f, rho - 1.0f, ux, uy, uz, Fx, Fy, Fz, true, P.omega);
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
        // keep the global band current for the rigid body and read-back
        band[7 * nb + b] = ftx;
        band[8 * nb + b] = fty;
        band[9 * nb + b] = ftz;
        if (THERMAL) {
            float g[QT];
#pragma unroll
            for (int l = 0; l < QT; l++) g[l] = St<T>::ld(GB + l * P.S + cell);
            const float Qt = fld[8 * slab_cells + c];
            const float Tc = fld[7 * slab_cells + c] + 0.5f * Qt;
            collide_heat(g, Tc, ux, uy, uz, Qt, P.omega_t);
#pragma unroll
            for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
            band[11 * nb + b] = Qt;
        }
    }

    // FP64 sums in a fixed order: per CTA, then over the cluster on CTA 0
    __shared__ double red[13][32];
    double sacc[13];
#pragma unroll
    for (int q = 0; q < 13; q++) sacc[q] = 0.0;
    const double xc0 = ds->body_xc[0], xc1 = ds->body_xc[1], xc2 = ds->body_xc[2];
    if (warp == 0) {
        for (int k = lane; k < nloc; k += 32) {
            const int m = r + CL * k;
            const double fx = mA[k], fy = mA[nloc_max + k], fz = mA[2 * nloc_max + k], hq = mA[3 * nloc_max + k];
            const double rx = mk.pos[m] - xc0, ry = mk.pos[n + m] - xc1, rz = mk.pos[2 * n + m] - xc2;
            sacc[0] += fx;
            sacc[1] += fy;
            sacc[2] += fz;
            sacc[3] += ry * fz - rz * fy;
            sacc[4] += rz * fx - rx * fz;
            sacc[5] += rx * fy - ry * fx;
            sacc[6] += hq;
        }
    }
    if (bp.free_body) {
        // fluid momentum inside the body (Kempe & Froehlich 2012): warp 1
        if (warp == 1) {
            for (int c = lane; c < my_cells; c += 32) {
                const int bz = z_lo + c / plane, rem = c % plane, by = rem / bsx, bx = rem % bsx;
                const int x = bx + o0, y = by + o1, z = bz + o2;
                if (x >= P.nx || y >= P.ny || z >= P.nz) continue;
                const double rx = (x + 1) - xc0, ry = (y + 1) - xc1, rz = (z + 1) - xc2;
                double a = bp.radius + 0.5 - sqrt(rx * rx + ry * ry + rz * rz);
                if (a <= 0.0) continue;
                if (a > 1.0) a = 1.0;
                const long long b = (long long)bz * plane + by * bsx + bx;
                const double rho = fld[c];
                const double ux = (double)fld[slab_cells + c] + 0.5 * band[4 * nb + b] / rho + fld[4 * slab_cells + c] / rho;
                const double uy = (double)fld[2 * slab_cells + c] + 0.5 * band[5 * nb + b] / rho + fld[5 * slab_cells + c] / rho;
                const double uz = (double)fld[3 * slab_cells + c] + 0.5 * band[6 * nb + b] / rho + fld[6 * slab_cells + c] / rho;
                sacc[7] += a * ux;
                sacc[8] += a * uy;
                sacc[9] += a * uz;
                sacc[10] += a * (ry * uz - rz * uy);
                sacc[11] += a * (rz * ux - rx * uz);
                sacc[12] += a * (rx * uy - ry * ux);
            }
        }
    }
    if (warp < 2) {
#pragma unroll
        for (int q = 0; q < 13; q++) red[q][lane] = (warp == 0 ? (q < 7 ? sacc[q] : 0.0) : 0.0);
    }
    __syncthreads();
    if (warp == 1) {
#pragma unroll
        for (int q = 7; q < 13; q++) red[q][lane] = sacc[q];
    }
    __syncthreads();
    if (tid < 13) {
        double v = 0.0;
        for (int i = 0; i < 32; i++) v += red[tid][i];
        part[tid] = v;
    }
    cluster.sync();
    __shared__ double tot[13];
    __shared__ double sh_dxc[3], sh_om[3], sh_v[3], sh_xc[3];
    if (r == 0) {
        if (tid < 13) {
            double v = 0.0;
            for (int q = 0; q < CL; q++) v += cluster.map_shared_rank(part, q)[tid];
            tot[tid] = v;
        }
    }
    cluster.sync();  // every remote read of the partial sums is done
    if (r != 0) return;
    if (tid == 0) {
        const long long step = ds->step;
        double *h = hist + (step % hist_cap) * 8;
        for (int k = 0; k < 7; k++) h[k] = tot[k];
        h[7] = (double)step;
        ds->step = step + 1;
        if (bp.free_body) {
            if (!ds->have_prev) {
                for (int k = 0; k < 6; k++) ds->internal_prev[k] = tot[7 + k];
                ds->have_prev = 1;
            }
            for (int a = 0; a < 3; a++) {
                const double dI = tot[7 + a] - ds->internal_prev[a];
                const double dL = tot[10 + a] - ds->internal_prev[3 + a];
                const double vn =
                    ((bp.dof >> a) & 1) ? ds->body_v[a] + (tot[a] + dI) / bp.mass + bp.gacc[a] : ds->body_v[a];
                const double om =
                    ((bp.dof >> (3 + a)) & 1) ? ds->body_om[a] + (tot[3 + a] + dL) / bp.inertia : ds->body_om[a];
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
            for (int k = 0; k < 6; k++) ds->internal_prev[k] = tot[7 + k];
            const int ns[3] = {P.nx, P.ny, P.nz};
            const int bs[3] = {P.bsx, P.bsy, P.bsz};
            for (int a = 0; a < 3; a++) {
                int o = (int)floor(sh_xc[a] - bp.radius) - 2;
                o = max(0, min(o, ns[a] - bs[a]));
                ds->band_o[a] = o;
            }
        }
    }
    if (!bp.free_body) return;
    __syncthreads();
    const double R = bp.radius;
    for (int m = tid; m < n; m += nthr) {
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

template <class T, bool THERMAL>
static size_t fused_smem(int slab_cells, int nloc_max) {
    constexpr int NF = THERMAL ? 9 : 7;
    size_t fl = (((size_t)NF * slab_cells + 5 * (size_t)nloc_max) * sizeof(float) + 15) / 16 * 16;
    return fl + (4 * (size_t)nloc_max + 16) * sizeof(double);
}

template <class T, bool THERMAL>
static cudaError_t plan_fused_t(const StepParams &P, int n_markers, FusedPlan &fp) {
    fp.enabled = 0;
    auto kern = k_ibm_fused<T, THERMAL>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    const int cands[3] = {16, 8, 4};
    for (int ci = 0; ci < 3; ci++) {
        const int CL = cands[ci];
        const int slab = (P.bsz + CL - 1) / CL;
        const int nloc_max = (n_markers + CL - 1) / CL;
        const size_t smem = fused_smem<T, THERMAL>(slab * P.bsx * P.bsy, nloc_max);
        if (smem > 200 * 1024) continue;
        if ((e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
            return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL, 1, 1);
        cfg.blockDim = dim3(512, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        e = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg);
        if (e != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (nclusters < 1) continue;
        fp.cl = CL;
        fp.slab = slab;
        fp.nloc_max = nloc_max;
        fp.smem = smem;
        fp.enabled = 1;
        return cudaSuccess;
    }
    return cudaSuccess;
}

cudaError_t plan_ibm_fused(int storage, bool thermal, const StepParams &P, int n_markers, FusedPlan &fp) {
    switch (storage) {
    case 0: return thermal ? plan_fused_t<float, true>(P, n_markers, fp) : plan_fused_t<float, false>(P, n_markers, fp);
    case 1: return thermal ? plan_fused_t<__half, true>(P, n_markers, fp) : plan_fused_t<__half, false>(P, n_markers, fp);
    case 2:
        return thermal ? plan_fused_t<__nv_bfloat16, true>(P, n_markers, fp)
                       : plan_fused_t<__nv_bfloat16, false>(P, n_markers, fp);
    }
    return cudaErrorInvalidValue;
}

template <class T, bool THERMAL>
static cudaError_t launch_fused_t(const IbmArgs &a, const FusedPlan &fp, void *B, void *GB, const BodyParams &bp,
                                  double *hist, long long hist_cap, int m_max, float fsign) {
    const int heat = a.thermal;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(fp.cl, 1, 1);
    cfg.blockDim = dim3(512, 1, 1);
    cfg.dynamicSmemBytes = fp.smem;
    cfg.stream = a.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = fp.cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_ibm_fused<T, THERMAL>, (T *)B, (T *)GB, *a.P, a.mk, a.ds, a.band, bp, hist,
                              hist_cap, m_max, fsign, fp.slab, fp.nloc_max, heat);
}

cudaError_t launch_ibm_fused(int storage, bool lattice_thermal, const IbmArgs &a, const FusedPlan &fp, void *B,
                             void *GB, const BodyParams &bp, double *hist, long long hist_cap, int m_max,
                             float fsign) {
    const bool th = lattice_thermal;
    switch (storage) {
    case 0:
        return th ? launch_fused_t<float, true>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign)
                  : launch_fused_t<float, false>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign);
    case 1:
        return th ? launch_fused_t<__half, true>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign)
                  : launch_fused_t<__half, false>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign);
    case 2:
        return th ? launch_fused_t<__nv_bfloat16, true>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign)
                  : launch_fused_t<__nv_bfloat16, false>(a, fp, B, GB, bp, hist, hist_cap, m_max, fsign);
    }
    return cudaErrorInvalidValue;
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
