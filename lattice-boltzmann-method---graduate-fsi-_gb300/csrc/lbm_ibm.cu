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

// Stencil of marker m: origin in band coordinates and the 4-point Peskin
// weights per axis (lbm.cpp:1095-1102).  The first interpolation of a step
// computes them from the marker position and stores them; the later passes
// and the spreadings of the step read them back.  Node s of the 4x4x4 block
// is (a, b, c) = (s & 3, (s >> 2) & 3, s >> 4); lane l holds s = l and l + 32,
// which share a and b.
struct Stencil {
    int bx0, by0, bz0;
    float kx, ky, kz0, kz1;  // this lane's weights: x of a, y of b, z of c and c + 2
};

__device__ __forceinline__ Stencil make_stencil(int m, int lane, const MarkerDev &mk, const DevState *ds,
                                                bool store) {
    const int n = mk.n;
    const double X = mk.pos[m], Y = mk.pos[n + m], Z = mk.pos[2 * n + m];
    const double flx = floor(X), fly = floor(Y), flz = floor(Z);
    const float fx = (float)(X - flx), fy = (float)(Y - fly), fz = (float)(Z - flz);
    Stencil st;
    // stencil node a: reference node i = floor(X) - 1 + a, device cell i - 1
    st.bx0 = (int)flx - 2 - ds->band_o[0];
    st.by0 = (int)fly - 2 - ds->band_o[1];
    st.bz0 = (int)flz - 2 - ds->band_o[2];
    const int a = lane & 3, b = (lane >> 2) & 3, c = lane >> 4;
    st.kx = peskin((float)(a - 1) - fx);
    st.ky = peskin((float)(b - 1) - fy);
    st.kz0 = peskin((float)(c - 1) - fz);
    st.kz1 = peskin((float)(c + 1) - fz);
    if (store) {
        if (lane == 0) {
            mk.sb[m] = st.bx0;
            mk.sb[n + m] = st.by0;
            mk.sb[2 * n + m] = st.bz0;
        }
        if (b == 0 && c == 0) mk.sw[a * n + m] = st.kx;
        if (a == 0 && c == 0) mk.sw[(4 + b) * n + m] = st.ky;
        if (a == 0 && b == 0) {
            mk.sw[(8 + c) * n + m] = st.kz0;
            mk.sw[(10 + c) * n + m] = st.kz1;
        }
    }
    return st;
}

__device__ __forceinline__ Stencil load_stencil(int m, int lane, const MarkerDev &mk) {
    const int n = mk.n;
    const int a = lane & 3, b = (lane >> 2) & 3, c = lane >> 4;
    Stencil st;
    st.bx0 = mk.sb[m];
    st.by0 = mk.sb[n + m];
    st.bz0 = mk.sb[2 * n + m];
    st.kx = mk.sw[a * n + m];
    st.ky = mk.sw[(4 + b) * n + m];
    st.kz0 = mk.sw[(8 + c) * n + m];
    st.kz1 = mk.sw[(10 + c) * n + m];
    return st;
}

// Interpolation at marker m (one warp) and the marker force of the next
// spreading: U_m = sum u delta with u = u_unf + Ft / (2 rho), rho_m on the
// first pass, F_m = 2 rho_m (U_des - U_m); the FP64 accumulators collect
// -F_m ds (the reference's Drag/Lift sums, lbm.cpp:1322-1323) and Q_m ds.
// After the warp sums, lanes 0-2 finish the x, y, z components and lane 3
// the heat source in parallel.
__device__ __forceinline__ void interp_marker(int m, int lane, const StepParams &P, const MarkerDev &mk,
                                              DevState *__restrict__ ds, const float *__restrict__ band, int first,
                                              int last, int thermal) {
    const int n = mk.n;
    const Stencil st = first ? make_stencil(m, lane, mk, ds, true) : load_stencil(m, lane, mk);
    const long long nb = P.nb;
    float su = 0.f, sv = 0.f, sw = 0.f, sr = 0.f, sT = 0.f;
    bool edge = false;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        const float wgt = st.kx * st.ky * (h == 0 ? st.kz0 : st.kz1);
        const int bx = st.bx0 + a, by = st.by0 + b, bz = st.bz0 + c;
        if ((unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            const float rho = 1.0f + band[q];
            const float hr = 0.5f / rho;
            su += wgt * (band[nb + q] + hr * from_fx(P.bandq[q]));
            sv += wgt * (band[2 * nb + q] + hr * from_fx(P.bandq[nb + q]));
            sw += wgt * (band[3 * nb + q] + hr * from_fx(P.bandq[2 * nb + q]));
            if (first) sr += wgt * rho;
            if (thermal) sT += wgt * (band[10 * nb + q] + 0.5f * from_fx(P.bandq[3 * nb + q]));
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
    if (lane == 0 && any_edge) atomicOr(&ds->status, ST_BAND_EDGE);
    if (first && lane == 0) mk.rho[m] = sr;
    const double dsv = mk.ds[m];
    double acc = 0.0;
    if (lane < 3) {
        const float sc = lane == 0 ? su : (lane == 1 ? sv : sw);
        const float rm = first ? sr : mk.rho[m];
        const float F = 2.0f * rm * (mk.udes[lane * n + m] - sc);
        mk.force[lane * n + m] = F;
        acc = mk.acc[lane * n + m] + -(double)F * dsv;
        if (!isfinite(F)) atomicOr(&ds->status, ST_NONFINITE_FORCE);
    } else if (lane == 3 && thermal) {
        const float Qm = 2.0f * (mk.tdes - sT);
        mk.force[3 * n + m] = Qm;
        acc = mk.acc[3 * n + m] + (double)Qm * dsv;
    }
    if (!last) {
        if (lane < 3 || (lane == 3 && thermal)) mk.acc[lane * n + m] = acc;
        return;
    }
    // the step's contribution of this marker, its torque about the body
    // centre included: the FP64 work is spread over every SM and the
    // one-block reduction only adds
    const double a0 = __shfl_sync(0xffffffffu, acc, 0);
    const double a1 = __shfl_sync(0xffffffffu, acc, 1);
    const double a2 = __shfl_sync(0xffffffffu, acc, 2);
    if (lane < 4) {
        mk.acc[(lane < 3 ? 4 + lane : 10) * n + m] = acc;
        mk.acc[lane * n + m] = 0.0;
    } else if (lane < 7) {
        const double rx = mk.pos[m] - ds->body_xc[0], ry = mk.pos[n + m] - ds->body_xc[1],
                     rz = mk.pos[2 * n + m] - ds->body_xc[2];
        const double t = lane == 4 ? ry * a2 - rz * a1 : (lane == 5 ? rz * a0 - rx * a2 : rx * a1 - ry * a0);
        mk.acc[(3 + lane) * n + m] = t;
    }
}

// Spreading of marker m (one warp): Ft(x) += F_m ds_m delta(x - X_m)
// (lbm.cpp:1331-1360), with the stencil the step's first interpolation
// stored.  The contributions go into the band's 64-bit fixed-point
// accumulators (to_fx): integer atomics, so every node's sum -- and the whole
// solve -- is the same in whatever order the markers' warps run.
__device__ __forceinline__ void spread_marker(int m, int lane, const StepParams &P, const MarkerDev &mk,
                                              const DevState *__restrict__ ds, float *__restrict__ band,
                                              int thermal) {
    const int n = mk.n;
    const Stencil st = load_stencil(m, lane, mk);
    const long long nb = P.nb;
    const float dsv = (float)mk.ds[m];
    const float Fx = mk.force[m] * dsv, Fy = mk.force[n + m] * dsv, Fz = mk.force[2 * n + m] * dsv;
    const float Qm = thermal ? mk.force[3 * n + m] * dsv : 0.0f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int s = lane + 32 * h;
        const int a = s & 3, b = (s >> 2) & 3, c = s >> 4;
        const float wgt = st.kx * st.ky * (h == 0 ? st.kz0 : st.kz1);
        const int bx = st.bx0 + a, by = st.by0 + b, bz = st.bz0 + c;
        if (wgt != 0.0f && (unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy &&
            (unsigned)bz < (unsigned)P.bsz) {
            const long long q = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
            unsigned long long *acc = reinterpret_cast<unsigned long long *>(P.bandq);
            atomicAdd(acc + q, (unsigned long long)to_fx(Fx * wgt));
            atomicAdd(acc + nb + q, (unsigned long long)to_fx(Fy * wgt));
            atomicAdd(acc + 2 * nb + q, (unsigned long long)to_fx(Fz * wgt));
            if (thermal) atomicAdd(acc + 3 * nb + q, (unsigned long long)to_fx(Qm * wgt));
        }
    }
}

// The IBM kernels run beside the far-region collide-stream launch, which
// leaves each SM 4096 registers: blocks of 64 threads with at most 64
// registers a thread fit there without waiting for its blocks to retire.
constexpr int kIbmThreads = 64;

__global__ void __launch_bounds__(kIbmThreads, 16) k_ibm_interp(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    DevState *__restrict__ ds, const float *__restrict__ band,
                                                    int first, int last, int thermal) {
    // launched early beside its predecessor (programmatic dependent
    // launch): wait for that grid's results before reading anything
    cudaGridDependencySynchronize();
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (m >= mk.n) return;  // whole warp leaves together
    interp_marker(m, threadIdx.x & 31, P, mk, ds, band, first, last, thermal);
}

__global__ void __launch_bounds__(kIbmThreads, 16) k_ibm_spread(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    const DevState *__restrict__ ds, float *__restrict__ band,
                                                    int thermal) {
    cudaGridDependencySynchronize();
    const int m = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (m >= mk.n) return;
    spread_marker(m, threadIdx.x & 31, P, mk, ds, band, thermal);
}

// One block.  Deterministic FP64 reductions: each thread sums a strided set
// in index order, then a fixed shared-memory tree.
// The one-block reduction kernel runs on its own, so it takes a full-size
// block: its per-thread loops over the markers and the band are four times
// shorter than with kIbmThreads.
constexpr int kFinishThreads = 256;
static_assert(kBodyBlocks <= kFinishThreads, "one partial per finishing thread");

__device__ __forceinline__ void block_tree(double (*red)[kFinishThreads], int nq, int t) {
    __syncthreads();
    for (int w = kFinishThreads / 2; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < nq; k++) red[k][t] += red[k][t + w];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kFinishThreads) k_ibm_finish(const __grid_constant__ StepParams P, MarkerDev mk,
                                                    DevState *__restrict__ ds, BodyParams bp,
                                                    const float *__restrict__ band, double *__restrict__ hist,
                                                    long long hist_cap) {
    __shared__ double red[7][kFinishThreads];
    __shared__ double sh_dxc[3], sh_om[3], sh_v[3], sh_xc[3], sh_f[7];  // written and read by thread 0
    const int t = threadIdx.x;
    const int n = mk.n;
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    // per-marker force, torque and heat of the step (the last interpolation)
    for (int m = t; m < n; m += kFinishThreads)
#pragma unroll
        for (int k = 0; k < 7; k++) s[k] += mk.acc[(4 + k) * (long long)n + m];
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
    // the internal-fluid momentum: the per-block partials of k_body_internal,
    // added in block order
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 6; k++) red[k][t] = t < kBodyBlocks ? mk.ipart[6 * t + k] : 0.0;
    block_tree(red, 6, t);
    if (t == 0) {
        if (!ds->have_prev) {
            for (int k = 0; k < 6; k++) ds->internal_prev[k] = red[k][0];
            for (int a = 0; a < 3; a++) {
                ds->body_v_prev[a] = ds->body_v[a];
                ds->body_om_prev[a] = ds->body_om[a];
            }
            ds->have_prev = 1;
        }
        // Newton-Euler, dt = 1, with the virtual mass of Schwarz, Kempe &
        // Froehlich (2015) on both sides (mv = iv = 0: plain explicit):
        //   (m + mv)(V' - V) = F_h + dI/dt + (rho_s - rho_f) V g + mv (V - V_prev)
        //   (I + iv)(W' - W) = T_h + dL/dt + iv (W - W_prev)
        for (int a = 0; a < 3; a++) {
            const double dI = red[a][0] - ds->internal_prev[a];
            const double dL = red[3 + a][0] - ds->internal_prev[3 + a];
            const double fb = (bp.mass - bp.vol) * bp.grav[a];
            const double vn = ((bp.dof >> a) & 1) ? ds->body_v[a] + (sh_f[a] + dI + fb +
                                                                    bp.mv * (ds->body_v[a] - ds->body_v_prev[a])) /
                                                                       (bp.mass + bp.mv)
                                                  : ds->body_v[a];
            const double om = ((bp.dof >> (3 + a)) & 1)
                                  ? ds->body_om[a] + (sh_f[3 + a] + dL + bp.iv * (ds->body_om[a] - ds->body_om_prev[a])) /
                                                         (bp.inertia + bp.iv)
                                  : ds->body_om[a];
            const double d = 0.5 * (ds->body_v[a] + vn);
            sh_dxc[a] = d;
            sh_v[a] = vn;
            sh_om[a] = om;
            sh_xc[a] = ds->body_xc[a] + d;
            ds->body_v_prev[a] = ds->body_v[a];
            ds->body_om_prev[a] = ds->body_om[a];
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
}

// Free body: fluid momentum and angular momentum inside the body after the
// forced collision, u_unf + F_b / (2 rho) + Ft / rho, with the volume
// fraction clamp(R + 1/2 - |x - xc|, 0, 1) (Kempe & Froehlich 2012), in
// FP64.  Block b sums its share of the band in index order (strided over its
// threads, then a fixed tree) into ipart[b]; k_ibm_finish adds the blocks in
// order.  Spread over kBodyBlocks SMs: GB300's FP64 rate on one SM made this
// sum the cost of the whole step.
__global__ void __launch_bounds__(kFinishThreads) k_body_internal(const __grid_constant__ StepParams P, MarkerDev mk,
                                                       const DevState *__restrict__ ds, BodyParams bp,
                                                       const float *__restrict__ band) {
    __shared__ double red[6][kFinishThreads];
    const int t = threadIdx.x;
    const long long nb = P.nb;
    const long long chunk = (nb + kBodyBlocks - 1) / kBodyBlocks;
    const long long b0 = blockIdx.x * chunk, b1 = min(nb, b0 + chunk);
    const double xc0 = ds->body_xc[0], xc1 = ds->body_xc[1], xc2 = ds->body_xc[2];
    double q[6] = {0, 0, 0, 0, 0, 0};
    for (long long b = b0 + t; b < b1; b += kFinishThreads) {
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
    if (t < 6) mk.ipart[6 * blockIdx.x + t] = red[t][0];
}

// Free body: move the markers with the body k_ibm_finish just advanced
// (x_c' = x_c + dx_c; r' = r + Omega' x r rescaled to R) and set their
// desired velocity V' + Omega' x r'.  One thread per marker.
__global__ void __launch_bounds__(128) k_body_markers(MarkerDev mk, const DevState *__restrict__ ds, BodyParams bp) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = mk.n;
    if (m >= n) return;
    const double R = bp.radius;
    const double xc[3] = {ds->body_xc[0], ds->body_xc[1], ds->body_xc[2]};
    const double dxc[3] = {ds->body_dxc[0], ds->body_dxc[1], ds->body_dxc[2]};
    const double om[3] = {ds->body_om[0], ds->body_om[1], ds->body_om[2]};
    const double v[3] = {ds->body_v[0], ds->body_v[1], ds->body_v[2]};
    const double r0 = mk.pos[m] - (xc[0] - dxc[0]);
    const double r1 = mk.pos[n + m] - (xc[1] - dxc[1]);
    const double r2 = mk.pos[2 * n + m] - (xc[2] - dxc[2]);
    double q0 = r0 + (om[1] * r2 - om[2] * r1);
    double q1 = r1 + (om[2] * r0 - om[0] * r2);
    double q2 = r2 + (om[0] * r1 - om[1] * r0);
    const double sc = R / sqrt(q0 * q0 + q1 * q1 + q2 * q2);
    q0 *= sc;
    q1 *= sc;
    q2 *= sc;
    mk.pos[m] = xc[0] + q0;
    mk.pos[n + m] = xc[1] + q1;
    mk.pos[2 * n + m] = xc[2] + q2;
    mk.udes[m] = (float)(v[0] + (om[1] * q2 - om[2] * q1));
    mk.udes[n + m] = (float)(v[1] + (om[2] * q0 - om[0] * q2));
    mk.udes[2 * n + m] = (float)(v[2] + (om[0] * q1 - om[1] * q0));
}

// One block: fixed-order FP64 sum of the per-block momentum-exchange
// partials of the listed blocks; record (Fx, Fy, Fz, step) with F the force
// on the solid cells (minus the exchange sums), then advance the step.
__global__ void __launch_bounds__(256) k_mea_finish(const float *__restrict__ part, const int *__restrict__ blocks,
                                                    int nblocks, double *__restrict__ ring, long long ring_cap,
                                                    DevState *__restrict__ ds, int advance) {
    __shared__ double red[3][256];
    const int t = threadIdx.x;
    double s[3] = {0.0, 0.0, 0.0};
    for (int i = t; i < nblocks; i += 256) {
        const long long b = blocks[i];
        for (int k = 0; k < 3; k++) s[k] += (double)part[3 * b + k];
    }
    for (int k = 0; k < 3; k++) red[k][t] = s[k];
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (t < w)
            for (int k = 0; k < 3; k++) red[k][t] += red[k][t + w];
        __syncthreads();
    }
    if (t == 0) {
        const long long step = ds->mea_step;
        double *r = ring + (step % ring_cap) * 4;
        for (int k = 0; k < 3; k++) r[k] = -red[k][0];
        r[3] = (double)step;
        if (advance) ds->mea_step = step + 1;
    }
}

cudaError_t launch_mea_finish(const float *part, const int *blocks, int nblocks, double *ring, long long ring_cap,
                              DevState *ds, int advance, cudaStream_t s) {
    k_mea_finish<<<1, 256, 0, s>>>(part, blocks, nblocks, ring, ring_cap, ds, advance);
    return cudaGetLastError();
}

// The interpolation/spreading chain of a step is a dozen short dependent
// grids.  With a.pdl each is launched with programmatic stream
// serialization: its launch is processed while its predecessor runs, and
// its blocks wait (cudaGridDependencySynchronize) for that grid's results.
// That shortens the chain, the FP32 sphere's critical path (31.9 k -> 34.5 k
// MLUPS); with FP16 storage, where the far-region streaming beside the chain
// is the critical path, it cost 3 % (40.7 k -> 39.6 k), so the host enables
// it for FP32 only.  Triggering the next grid early from the top of each
// kernel was worse for both (33.8 k, 38.9 k): its waiting blocks hold SM
// slots.
static cudaLaunchConfig_t pdl_config(dim3 grid, dim3 block, cudaStream_t s, cudaLaunchAttribute *attr, int pdl) {
    cudaLaunchConfig_t c = {};
    c.gridDim = grid;
    c.blockDim = block;
    c.dynamicSmemBytes = 0;
    c.stream = s;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = attr;
    c.numAttrs = pdl ? 1 : 0;
    return c;
}

cudaError_t launch_ibm_interp(const IbmArgs &a, int first, int last) {
    const int threads = kIbmThreads;
    const long long blocks = ((long long)a.mk.n * 32 + threads - 1) / threads;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t c = pdl_config(dim3((unsigned)blocks), dim3(threads), a.stream, attr, a.pdl);
    return cudaLaunchKernelEx(&c, k_ibm_interp, *a.P, a.mk, a.ds, (const float *)a.band, first, last, a.thermal);
}

cudaError_t launch_ibm_spread(const IbmArgs &a) {
    const int threads = kIbmThreads;
    const long long blocks = ((long long)a.mk.n * 32 + threads - 1) / threads;
    cudaLaunchAttribute attr[1];
    cudaLaunchConfig_t c = pdl_config(dim3((unsigned)blocks), dim3(threads), a.stream, attr, a.pdl);
    return cudaLaunchKernelEx(&c, k_ibm_spread, *a.P, a.mk, (const DevState *)a.ds, a.band, a.thermal);
}

cudaError_t launch_ibm_finish(const IbmArgs &a, const BodyParams &bp, double *hist, long long hist_cap) {
    if (bp.free_body) k_body_internal<<<kBodyBlocks, kFinishThreads, 0, a.stream>>>(*a.P, a.mk, a.ds, bp, a.band);
    k_ibm_finish<<<1, kFinishThreads, 0, a.stream>>>(*a.P, a.mk, a.ds, bp, a.band, hist, hist_cap);
    if (bp.free_body) k_body_markers<<<(a.mk.n + 127) / 128, 128, 0, a.stream>>>(a.mk, a.ds, bp);
    return cudaGetLastError();
}

}  // namespace lbmk
