// lbm_energy3d.cu -- the reference's ENERGY model on D3Q19 (#define ENERGY
// without D2Q9; its Rayleigh_Benard case, LBM.h:222-242, lbm.cpp:1585-1643):
// temperature populations g on the flow lattice with viscous heating,
// Dirichlet (TYPE_T), Neumann (TYPE_Q) and adiabatic walls, and the
// Boussinesq force that MacroProp refreshes on every cell (lbm.cpp:803-805).
//
// The device grid is the reference's ghost-inclusive one, (Nx+2)(Ny+2)(Nz+2)
// cells with its periodic modulo over the whole grid, so every wall rule
// reads the cells the reference reads.  f and g are FP32, stored shifted
// (f - w, g - w T_ref) in [19][S] arrays, two of each (pull scheme).
//
// The reference applies its thermal wall rules inside a serial push
// (lbm.cpp:240-289): a Neumann wall's T (Determine_Twall_Neumann,
// lbm.cpp:983-1028) sums the cell's g while neighbours are still pushing,
// and is written into wall cells that Determine_Wall_Temperature
// (lbm.cpp:965-981) of cells visited later reads for their Dirichlet links.
// Every value such a read can see is known before the sweep: the wall T a
// Neumann cell forms depends only on the previous collision and on its own
// previous g.  So the host replays the visiting order once (build_records)
// and gives each wall-adjacent fluid cell a record: its link masks, the
// wall velocity of each phase, and for each solid neighbour the cell whose
// Neumann write it sees (or none, then the wall's own T).  Per step a
// pre-pass (k_e3_walls) forms the Neumann cells' T_w; the step kernel
// (k_e3_bulk for the other fluid cells; k_e3_rgather and k_e3_rcollide for
// the records) pulls, applies the wall rules, takes the moments, refreshes
// the force and collides.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_collide.cuh"
#include "lbm_device.cuh"

void lbm_set_last_error(const std::string &m);

namespace {
using namespace lbmk;

constexpr int kSlots = 18;       // solid neighbours a cell can have
constexpr int kTypeF = 0, kTypeS = 1, kTypeT = 6, kTypeQ = 7;
constexpr int kBlock = 256;
constexpr int kRecBlock = 64;  // the record kernels: latency-bound, spread over every SM

// A fluid cell with at least one solid neighbour.  Links are indexed by the
// pulled direction p (source c - c_p); the reference's push direction of
// that wall link is opp(p).  Its Dirichlet links' wall T is the mean over
// its solid neighbours: the ones no Neumann write reaches are summed once
// (ssum); the others ("dynamic") are listed with the record whose write the
// cell sees and the push index of the cell's own write.
struct E3Rec {
    int cell;
    int i, j, k;             // its coordinates
    uint32_t bb;             // links whose source is solid
    uint32_t dir, neu, adi;  // ... of type_Energy TYPE_T, TYPE_Q, any other
    int ndyn;                // dynamic solid neighbours
    float inv_nsol;          // 1 / solid neighbours
    float ssum[2];           // T of the other solid neighbours: set-up (streaming 1), MacroProp's (later)
    float uw[3][3];          // Determine_Wall_Velocity at streaming 1, 2, and from 3 on
    int dwriter[kSlots];     // record whose Neumann push last wrote its T before this cell; -1 none
    float dt[2][kSlots];     // its own T, as ssum
    uint8_t down[kSlots];    // push index at which this cell itself writes its T; 255 never
};

// The solid neighbours of a record while the host builds it.
struct E3Slots {
    int nsol = 0;
    long long cell[kSlots];
    int writer[kSlots];
    float tsol[2][kSlots];
    uint8_t own[kSlots];
};

// The records on the device, one array per field (a warp's load of a field
// reads 32 consecutive records).
struct E3Recs {
    const int *cell, *ci, *cj, *ck;
    const uint32_t *bb, *dir, *neu;
    const int *ndyn;
    const float *inv_nsol;
    const float *ssum;     // [2][nrec]
    const float *uw;       // [3 phases][3][nrec]
    const int *dwriter;    // [kSlots][nrec]
    const float *dt;       // [2][kSlots][nrec]
    const uint8_t *down;   // [kSlots][nrec]
};

// rec_of: a record index, or one of these
constexpr int kSolid = -2, kBulk = -1, kBulkWrap = -3;

struct E3Params {
    int NX, NY, NZ;
    long long N, S;
    int offs[Q];  // source of link l: c - offs[l] away from the grid's faces
    int nrec;
    float omega, inv_tau_g, tg_fac, inv_cp, two_nu, s_fac, T_ref;
    float gbeta, T_star;
    int buoy, forced;
};

// The source c - c_l of cell (i, j, k) under the reference's periodic
// modulo over the whole grid (lbm.cpp:252-255); its coordinates in a, b, d.
__device__ __forceinline__ int wrap_src(int i, int j, int k, int l, const E3Params &P, int &a, int &b, int &d) {
    a = i - cx(l);
    b = j - cy(l);
    d = k - cz(l);
    a += a < 0 ? P.NX : (a >= P.NX ? -P.NX : 0);
    b += b < 0 ? P.NY : (b >= P.NY ? -P.NY : 0);
    d += d < 0 ? P.NZ : (d >= P.NZ ? -P.NZ : 0);
    return a + P.NX * (b + P.NY * d);
}
__device__ __forceinline__ int wrap_src(int i, int j, int k, int l, const E3Params &P) {
    int a, b, d;
    return wrap_src(i, j, k, l, P, a, b, d);
}

// 1 + 3x + 4.5x^2 - 1.5uu (+ 4.5x(x^2 - uu) for the cubic form), x = c.u
__device__ __forceinline__ float p2m1(float x, float uu) { return 3.0f * x + 4.5f * x * x - 1.5f * uu; }
__device__ __forceinline__ float p3m1(float x, float uu) { return p2m1(x, uu) + 4.5f * x * (x * x - uu); }

// The D3Q19 link vectors as 2-bit fields (c + 1) of one word per axis, for a
// link index that differs across the lanes of a warp.
__host__ __device__ constexpr unsigned long long pack_axis(int a) {
    unsigned long long v = 0;
    for (int l = 0; l < Q; l++) v |= (unsigned long long)((a == 0 ? cx(l) : (a == 1 ? cy(l) : cz(l))) + 1) << (2 * l);
    return v;
}
__device__ __forceinline__ int lane_c(unsigned long long packed, int l) { return (int)((packed >> (2 * l)) & 3ull) - 1; }
__device__ __forceinline__ float lane_w(int l) { return l == 0 ? 1.0f / 3.0f : (l < 7 ? 1.0f / 18.0f : 1.0f / 36.0f); }
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Determine_Twall_Neumann for every record with Neumann links, one warp a
// record and one lane a link: the normal is the mean direction of the links
// from walls (cdotn_pos); the other links contribute this sweep's pulled
// value where the reference's push (i outer, k inner) visits their source
// before the cell -- and for the rest link --, else the previous sweep's,
// kept in gold; the wall links the equilibrium at T = 1 of the cell's
// density (previous MacroProp) and the wall velocity.  With j.n = 0
// (LBM.h's j_dot_n): T_w = -sum_other g c.n / sum_wall geq c.n, the sums
// over the lanes.  keep: store this sweep's pulled values for the next
// sweep's stale links.
constexpr int kWallBlock = 128;
__global__ void __launch_bounds__(kWallBlock) k_e3_walls(const float *__restrict__ GA, const float4 *__restrict__ aux,
                                                         const __grid_constant__ E3Recs R, float *__restrict__ gold,
                                                         float *__restrict__ tw, const __grid_constant__ E3Params P,
                                                         int phase, int keep) {
    const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (r >= P.nrec) return;  // whole warps
    if (!R.neu[r]) return;    // uniform over the warp
    constexpr unsigned long long PX = pack_axis(0), PY = pack_axis(1), PZ = pack_axis(2);
    const int lane = threadIdx.x & 31;
    const bool act = lane < Q;
    const int p = act ? lane : 0;
    const int ex = lane_c(PX, p), ey = lane_c(PY, p), ez = lane_c(PZ, p);
    const uint32_t bb = R.bb[r];
    const bool wl = act && ((bb >> p) & 1u);
    const int c = R.cell[r], i = R.ci[r], j = R.cj[r], k = R.ck[r];
    // the other links' loads first
    float vnew = 0.0f, vold = 0.0f;
    bool fresh = true;
    int s = 0;
    if (act && !wl) {
        int a = i - ex, b = j - ey, d = k - ez;
        a += a < 0 ? P.NX : (a >= P.NX ? -P.NX : 0);
        b += b < 0 ? P.NY : (b >= P.NY ? -P.NY : 0);
        d += d < 0 ? P.NZ : (d >= P.NZ ? -P.NZ : 0);
        s = a + P.NX * (b + P.NY * d);
        fresh = p == 0 || a < i || (a == i && (b < j || (b == j && d < k)));
        vnew = GA[p * P.S + s];
        if (!fresh) vold = gold[(long long)p * P.nrec + r];
    }
    const float u0 = R.uw[(3 * phase) * P.nrec + r], u1 = R.uw[(3 * phase + 1) * P.nrec + r],
                u2 = R.uw[(3 * phase + 2) * P.nrec + r];
    const float rho = 1.0f + aux[c].x;
    // the normal: the mean wall-link direction (sums of small integers, exact)
    const float nw = warp_sum(wl ? 1.0f : 0.0f);
    const float n0 = warp_sum(wl ? (float)ex : 0.0f) / nw, n1 = warp_sum(wl ? (float)ey : 0.0f) / nw,
                n2 = warp_sum(wl ? (float)ez : 0.0f) / nw;
    const float cn = ex * n0 + ey * n1 + ez * n2;
    float wall = 0.0f, other = 0.0f;
    if (wl) {
        const float uu = u0 * u0 + u1 * u1 + u2 * u2;
        const float x = ex * u0 + ey * u1 + ez * u2;
        wall = lane_w(p) * (1.0f + p3m1(x, uu)) * cn;
    } else if (act) {
        other = ((fresh ? vnew : vold) + lane_w(p) * P.T_ref) * cn;
    }
    wall = warp_sum(wall);
    other = warp_sum(other);
    if (lane == 0) tw[r] = -other / (rho * wall);
    if (keep && act && !wl && !fresh) gold[(long long)p * P.nrec + r] = vnew;
}

// The same, one thread a record: the form for grids whose wall records are a
// small share, where it does not crowd the bulk kernel beside it.
// Determine_Twall_Neumann for every record with Neumann links: the normal is
// the mean direction of the links from walls (cdotn_pos); the other links
// contribute this sweep's pulled value where the reference's push (i outer,
// k inner) visits their source before the cell -- and for the rest link --,
// else the previous sweep's, kept in gold; the wall links the equilibrium
// at T = 1 of the cell's density (previous MacroProp) and the wall velocity.
// With j.n = 0 (LBM.h's j_dot_n): T_w = -sum_other g c.n / sum_wall geq c.n.
// keep: store this sweep's pulled values for the next sweep.
__global__ void __launch_bounds__(kRecBlock) k_e3_walls_t(const float *__restrict__ GA, const float4 *__restrict__ aux,
                                                     const __grid_constant__ E3Recs R, float *__restrict__ gold,
                                                     float *__restrict__ tw, const __grid_constant__ E3Params P,
                                                     int phase, int keep) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.nrec) return;
    if (!R.neu[r]) return;
    const uint32_t bb = R.bb[r];
    const int c = R.cell[r], i = R.ci[r], j = R.cj[r], k = R.ck[r];
    float n0 = 0.0f, n1 = 0.0f, n2 = 0.0f;
    int np = 0;
#pragma unroll
    for (int p = 0; p < Q; p++)
        if ((bb >> p) & 1u) {
            n0 += cx(p);
            n1 += cy(p);
            n2 += cz(p);
            np++;
        }
    const float inv_np = 1.0f / (float)np;
    n0 *= inv_np;
    n1 *= inv_np;
    n2 *= inv_np;
    const float u0 = R.uw[(3 * phase) * P.nrec + r], u1 = R.uw[(3 * phase + 1) * P.nrec + r],
                u2 = R.uw[(3 * phase + 2) * P.nrec + r];
    const float uu = u0 * u0 + u1 * u1 + u2 * u2;
    // every load first (the kept values are rewritten below)
    float v[Q];
    uint32_t fresh = 0u;
#pragma unroll
    for (int p = 0; p < Q; p++) {
        if ((bb >> p) & 1u) continue;
        int si, sj, sk;
        const int s = wrap_src(i, j, k, p, P, si, sj, sk);
        const bool fr = p == 0 || si < i || (si == i && (sj < j || (sj == j && sk < k)));
        v[p] = fr ? GA[p * P.S + s] : gold[(long long)p * P.nrec + r];
        if (fr) fresh |= 1u << p;
    }
    const float rho = 1.0f + aux[c].x;
    float other = 0.0f, wall = 0.0f;
#pragma unroll
    for (int p = 0; p < Q; p++) {
        const float cn = cx(p) * n0 + cy(p) * n1 + cz(p) * n2;
        if ((bb >> p) & 1u) {
            const float x = cx(p) * u0 + cy(p) * u1 + cz(p) * u2;
            wall += wf(p) * (1.0f + p3m1(x, uu)) * cn;
        } else {
            other += (v[p] + wf(p) * P.T_ref) * cn;
        }
    }
    tw[r] = -other / (rho * wall);
    if (!keep) return;
    // this sweep's pulled values for the next sweep's stale links
#pragma unroll
    for (int p = 0; p < Q; p++) {
        if (((bb | fresh) >> p) & 1u) continue;
        gold[(long long)p * P.nrec + r] = GA[p * P.S + wrap_src(i, j, k, p, P)];
    }
}

// MacroProp and the collision of one fluid cell whose pulled populations
// are f and g (lbm.cpp:657-806, 91-177).  gather = 0: the first collision,
// on the set-up state (no streaming before it).  aux[c] = (rho - 1, u) of
// the last MacroProp (the previous collision's); aux2[c] = (Phi of the
// previous collision, the force of the last MacroProp).  MacroProp:
// u = (j + F/2) / rho with the force of the previous MacroProp, T = sum g,
// q = sum g c, then F_y = g beta (T - T*) when the buoyancy is on.  ConvLBM:
// f by BGK + Guo with that force; g by BGK with the viscous-heating source
// F_l = w Phi / cp (1 + c.u (tau_g - 1/2) / (cs2 tau_g)) and half its change
// since the previous collision.
__device__ __forceinline__ void macro_collide(int c, float f[Q], float g[Q], float4 h1, float4 h2,
                                              const E3Params &P, float *__restrict__ B, float *__restrict__ GB,
                                              float4 *__restrict__ aux, float4 *__restrict__ aux2,
                                              uint32_t *__restrict__ status, float *__restrict__ mom, int gather,
                                              int export_only) {
    float drho, jx, jy, jz;
    moments_pairs(f, drho, jx, jy, jz);
    float dT = 0.0f, qx = 0.0f, qy = 0.0f, qz = 0.0f;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        dT += g[l];
        if (cx(l)) qx += cx(l) * g[l];
        if (cy(l)) qy += cy(l) * g[l];
        if (cz(l)) qz += cz(l) * g[l];
    }
    const float rho = 1.0f + drho;
    const float inv = 1.0f / rho;
    // before the first MacroProp the collision takes the set-up state:
    // u = j / rho, T = sum g / rho (the initial g sum to rho T)
    const float hf = gather ? 0.5f : 0.0f;
    const float ux = (jx + hf * h2.y) * inv, uy = (jy + hf * h2.z) * inv, uz = (jz + hf * h2.w) * inv;
    const float Tc = gather ? P.T_ref + dT : (P.T_ref + dT) * inv;
    // rho T - T_ref
    const float Tdiff = gather ? dT + drho * Tc : dT;
    float Fx = h2.y, Fy = h2.z, Fz = h2.w;
    if (gather && P.buoy) Fy = P.gbeta * (Tc - P.T_star);
    if (!(rho > 0.0f && rho < 100.0f)) raise_status(status, ST_RHO_RANGE);
    if (!(Tc > 0.0f && Tc < 100.0f)) raise_status(status, ST_T_RANGE);
    if (mom != nullptr) {
        mom[c] = rho;
        mom[P.N + c] = ux;
        mom[2 * P.N + c] = uy;
        mom[3 * P.N + c] = uz;
        mom[4 * P.N + c] = Tc;
        mom[5 * P.N + c] = qx;  // sum g c: the shift w T_ref carries no momentum
        mom[6 * P.N + c] = qy;
        mom[7 * P.N + c] = qz;
    }
    if (export_only) return;
    const float usq = ux * ux + uy * uy + uz * uz;
    float sxx = 0.0f, syy = 0.0f, szz = 0.0f, sxy = 0.0f, sxz = 0.0f, syz = 0.0f;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float fne = f[l] - wf(l) * (drho + rho * p3m1(cu, usq));
        sxx += (float)(cx(l) * cx(l)) * fne;
        syy += (float)(cy(l) * cy(l)) * fne;
        szz += (float)(cz(l) * cz(l)) * fne;
        sxy += (float)(cx(l) * cy(l)) * fne;
        sxz += (float)(cx(l) * cz(l)) * fne;
        syz += (float)(cy(l) * cz(l)) * fne;
    }
    const float sk = P.s_fac * inv;
    sxx *= sk;
    syy *= sk;
    szz *= sk;
    sxy *= sk;
    sxz *= sk;
    syz *= sk;
    const float phi =
        P.two_nu * rho * (sxx * sxx + syy * syy + szz * szz + 2.0f * (sxy * sxy + sxz * sxz + syz * syz));
    collide_flow(f, drho, ux, uy, uz, Fx, Fy, Fz, P.forced != 0, P.omega);
    const float a = phi * P.inv_cp, ap = h2.x * P.inv_cp;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float cup = cx(l) * h1.y + cy(l) * h1.z + cz(l) * h1.w;
        const float Fl = wf(l) * a * (1.0f + cu * P.tg_fac);
        const float Fb = wf(l) * ap * (1.0f + cup * P.tg_fac);
        const float geq = wf(l) * (Tdiff + rho * Tc * p3m1(cu, usq));
        g[l] = g[l] - (g[l] - geq) * P.inv_tau_g + Fl + 0.5f * (Fl - Fb);
    }
    aux[c] = make_float4(drho, ux, uy, uz);
    aux2[c] = make_float4(phi, Fx, Fy, Fz);
#pragma unroll
    for (int l = 0; l < Q; l++) {
        B[l * P.S + c] = f[l];
        GB[l * P.S + c] = g[l];
    }
}

// The fluid cells without a solid neighbour (solid cells and wall records
// idle): a plain pull, offsets away from the grid's faces, the reference's
// periodic modulo on them.
__global__ void __launch_bounds__(kBlock) k_e3_bulk(const float *__restrict__ A, float *__restrict__ B,
                                                    const float *__restrict__ GA, float *__restrict__ GB,
                                                    float4 *__restrict__ aux, float4 *__restrict__ aux2,
                                                    const int *__restrict__ rec_of, const __grid_constant__ E3Params P,
                                                    uint32_t *__restrict__ status, float *__restrict__ mom,
                                                    int gather, int export_only) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.N) return;
    const int ro = rec_of[c];
    if (ro != kBulk && ro != kBulkWrap) return;
    const float4 h1 = aux[c], h2 = aux2[c];
    float f[Q], g[Q];
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            f[l] = A[l * P.S + c];
            g[l] = GA[l * P.S + c];
        }
    } else if (ro == kBulk) {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            const int s = c - P.offs[l];
            f[l] = A[l * P.S + s];
            g[l] = GA[l * P.S + s];
        }
    } else {
        const int i = c % P.NX, j = (c / P.NX) % P.NY, k = c / (P.NX * P.NY);
#pragma unroll
        for (int l = 0; l < Q; l++) {
            const int s = wrap_src(i, j, k, l, P);
            f[l] = A[l * P.S + s];
            g[l] = GA[l * P.S + s];
        }
    }
    macro_collide(c, f, g, h1, h2, P, B, GB, aux, aux2, status, mom, gather, export_only);
}

// The wall records' pull, one warp a record and one lane a link, into the
// scratch array (f then g, [2 Q][records]): the reference's wall rules
// (lbm.cpp:266-288).  f: bounce-back with Determine_Wall_Velocity; g:
// Dirichlet anti-bounce-back at Determine_Wall_Temperature's T as the sweep
// has left the solid neighbours (the lanes load the dynamic neighbours'
// values; a link's own-write corrections come by shuffles), Neumann the
// equilibrium of the pre-pass's T_w, adiabatic the kept initial value.
__global__ void __launch_bounds__(kWallBlock) k_e3_rgather(const float *__restrict__ A, const float *__restrict__ GA,
                                                           const float4 *__restrict__ aux,
                                                           const __grid_constant__ E3Recs R,
                                                           const float *__restrict__ gold, const float *__restrict__ tw,
                                                           float *__restrict__ scr, const __grid_constant__ E3Params P,
                                                           int phase) {
    const int r = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    if (r >= P.nrec) return;  // whole warps
    constexpr unsigned long long PX = pack_axis(0), PY = pack_axis(1), PZ = pack_axis(2);
    const int lane = threadIdx.x & 31;
    const bool act = lane < Q;
    const int p = act ? lane : 0;
    const int ex = lane_c(PX, p), ey = lane_c(PY, p), ez = lane_c(PZ, p);
    const int c = R.cell[r], i = R.ci[r], j = R.cj[r], k = R.ck[r];
    const uint32_t bb = R.bb[r], dir = R.dir[r], neu = R.neu[r];
    // launched early behind the pre-pass (programmatic dependent launch):
    // the record's fields above never change; wait before the populations
    cudaGridDependencySynchronize();
    const bool wl = act && ((bb >> p) & 1u);
    float fv = 0.0f, gv = 0.0f;
    if (act && !wl) {
        int sa = i - ex, sb = j - ey, sc = k - ez;
        sa += sa < 0 ? P.NX : (sa >= P.NX ? -P.NX : 0);
        sb += sb < 0 ? P.NY : (sb >= P.NY ? -P.NY : 0);
        sc += sc < 0 ? P.NZ : (sc >= P.NZ ? -P.NZ : 0);
        const int src = sa + P.NX * (sb + P.NY * sc);
        fv = A[p * P.S + src];
        gv = GA[p * P.S + src];
    }
    const int ph = phase == 0 ? 0 : 1;
    const float tw_own = neu ? tw[r] : 0.0f;
    // the dynamic solid neighbours' T as this cell's push starts (the last
    // Neumann write before the cell, or the wall's own T), one lane each
    const int ndyn = R.ndyn[r];
    float vdl = 0.0f;
    int dl = 255;
    if (lane < ndyn) {
        const int w = R.dwriter[lane * P.nrec + r];
        vdl = w >= 0 ? tw[w] : R.dt[(ph * kSlots + lane) * P.nrec + r];
        dl = R.down[lane * P.nrec + r];
    }
    const float vsum = R.ssum[ph * P.nrec + r] + warp_sum(vdl);
    // the reference's push direction of this link, towards the wall
    const int q = p == 0 ? 0 : ((p & 1) ? p + 1 : p - 1);
    // the neighbours this cell's own Neumann links wrote before push index q
    float corr = 0.0f;
    for (int m = 0; m < ndyn; m++) {
        const float vm = __shfl_sync(0xffffffffu, vdl, m);
        const int dm = __shfl_sync(0xffffffffu, dl, m);
        if (dm < q) corr += tw_own - vm;
    }
    if (wl) {
        const float u0 = R.uw[(3 * phase) * P.nrec + r], u1 = R.uw[(3 * phase + 1) * P.nrec + r],
                    u2 = R.uw[(3 * phase + 2) * P.nrec + r];
        const float uu = u0 * u0 + u1 * u1 + u2 * u2;
        const float rho_p = 1.0f + aux[c].x;
        const float w = lane_w(p);
        const float x = -(ex * u0 + ey * u1 + ez * u2);  // c_q . u_w
        // f_opp(q) = f*_q - 2 w (u_w . c_q) / cs2 (lbm.cpp:273-274)
        fv = A[q * P.S + c] - 6.0f * w * x;
        if ((dir >> p) & 1u) {
            const float Tw = (vsum + corr) * R.inv_nsol[r];
            // -g*_q + 2 geq_q(rho, T_w, u_w) (lbm.cpp:277-280)
            gv = 2.0f * w * (rho_p * Tw * (1.0f + p3m1(x, uu)) - P.T_ref) - GA[q * P.S + c];
        } else if ((neu >> p) & 1u) {
            // w rho T_w times the second-order shape of the wall (lbm.cpp:281-288)
            gv = w * (rho_p * tw_own * (1.0f + p2m1(x, uu)) - P.T_ref);
        } else {
            gv = gold[(long long)p * P.nrec + r];  // never written: the initial value
        }
    }
    if (act) {
        scr[(long long)p * P.nrec + r] = fv;
        scr[(long long)(Q + p) * P.nrec + r] = gv;
    }
}

// MacroProp and the collision of the wall records, one thread each, from the
// gathered populations (the first collision: from the set-up state, whose g
// become the kept initial values).
__global__ void __launch_bounds__(kRecBlock) k_e3_rcollide(const float *__restrict__ A, float *__restrict__ B,
                                                           const float *__restrict__ GA, float *__restrict__ GB,
                                                           float4 *__restrict__ aux, float4 *__restrict__ aux2,
                                                           const __grid_constant__ E3Recs R, float *__restrict__ gold,
                                                           const float *__restrict__ scr,
                                                           const __grid_constant__ E3Params P,
                                                           uint32_t *__restrict__ status, float *__restrict__ mom,
                                                           int gather, int export_only) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.nrec) return;
    const int c = R.cell[r];
    cudaGridDependencySynchronize();  // behind the gather (programmatic dependent launch)
    const float4 h1 = aux[c], h2 = aux2[c];
    float f[Q], g[Q];
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            f[l] = A[l * P.S + c];
            g[l] = GA[l * P.S + c];
        }
        if (!export_only) {
#pragma unroll
            for (int l = 0; l < Q; l++) gold[(long long)l * P.nrec + r] = g[l];
        }
    } else {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            f[l] = scr[(long long)l * P.nrec + r];
            g[l] = scr[(long long)(Q + l) * P.nrec + r];
        }
    }
    macro_collide(c, f, g, h1, h2, P, B, GB, aux, aux2, status, mom, gather, export_only);
}

// The wall records in one pass, one thread each (the form for grids whose
// records are a small share): the pull with the reference's wall
// rules (lbm.cpp:266-288).  f: bounce-back with Determine_Wall_Velocity;
// g: Dirichlet anti-bounce-back at Determine_Wall_Temperature's T as the
// sweep has left the solid neighbours, Neumann the equilibrium of the
// pre-pass's T_w, adiabatic the kept initial value.
__global__ void __launch_bounds__(kRecBlock) k_e3_rec(const float *__restrict__ A, float *__restrict__ B,
                                                   const float *__restrict__ GA, float *__restrict__ GB,
                                                   float4 *__restrict__ aux, float4 *__restrict__ aux2,
                                                   const __grid_constant__ E3Recs R, float *__restrict__ gold,
                                                   const float *__restrict__ tw, const __grid_constant__ E3Params P,
                                                   uint32_t *__restrict__ status, float *__restrict__ mom, int gather,
                                                   int phase, int export_only) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P.nrec) return;
    const int c = R.cell[r];
    const float4 h1 = aux[c], h2 = aux2[c];
    float f[Q], g[Q];
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            f[l] = A[l * P.S + c];
            g[l] = GA[l * P.S + c];
        }
        if (!export_only) {
#pragma unroll
            for (int l = 0; l < Q; l++) gold[(long long)l * P.nrec + r] = g[l];
        }
    } else {
        const int i = R.ci[r], j = R.cj[r], k = R.ck[r];
        const uint32_t bb = R.bb[r], dir = R.dir[r], neu = R.neu[r];
        const float u0 = R.uw[(3 * phase) * P.nrec + r], u1 = R.uw[(3 * phase + 1) * P.nrec + r],
                    u2 = R.uw[(3 * phase + 2) * P.nrec + r];
        const float uu = u0 * u0 + u1 * u1 + u2 * u2;
        const float rho_p = 1.0f + h1.x;
        const float tw_own = neu ? tw[r] : 0.0f;
        const int ph = phase == 0 ? 0 : 1;
        // the dynamic solid neighbours' T as this cell's push starts: the
        // last Neumann write before the cell, or the wall's own T
        float vd[kSlots];
        float vsum = R.ssum[ph * P.nrec + r];
        const int ndyn = R.ndyn[r];
#pragma unroll 6
        for (int m = 0; m < ndyn; m++) {
            const int w = R.dwriter[m * P.nrec + r];
            vd[m] = w >= 0 ? tw[w] : R.dt[(ph * kSlots + m) * P.nrec + r];
        }
#pragma unroll 1
        for (int m = 0; m < ndyn; m++) vsum += vd[m];
#pragma unroll
        for (int p = 0; p < Q; p++) {
            if (!((bb >> p) & 1u)) {
                const int s = wrap_src(i, j, k, p, P);
                f[p] = A[p * P.S + s];
                g[p] = GA[p * P.S + s];
                continue;
            }
            const int q = opp(p);  // the reference's push direction, towards the wall
            const float x = cx(q) * u0 + cy(q) * u1 + cz(q) * u2;
            // f_opp(q) = f*_q - 2 w (u_w . c_q) / cs2 (lbm.cpp:273-274)
            f[p] = A[q * P.S + c] - 6.0f * wf(q) * x;
            if ((dir >> p) & 1u) {
                // Determine_Wall_Temperature at this point of the push: the
                // neighbours this cell's own Neumann links wrote earlier in
                // its push hold its T_w
                float Tsum = vsum;
#pragma unroll 1
                for (int m = 0; m < ndyn; m++)
                    if (R.down[m * P.nrec + r] < q) Tsum += tw_own - vd[m];
                const float Tw = Tsum * R.inv_nsol[r];
                // -g*_q + 2 geq_q(rho, T_w, u_w) (lbm.cpp:277-280)
                g[p] = 2.0f * wf(q) * (rho_p * Tw * (1.0f + p3m1(x, uu)) - P.T_ref) - GA[q * P.S + c];
            } else if ((neu >> p) & 1u) {
                // w rho T_w times the second-order shape of the wall (lbm.cpp:281-288)
                g[p] = wf(q) * (rho_p * tw_own * (1.0f + p2m1(x, uu)) - P.T_ref);
            } else {
                g[p] = gold[(long long)p * P.nrec + r];  // never written: the initial value
            }
        }
    }
    macro_collide(c, f, g, h1, h2, P, B, GB, aux, aux2, status, mom, gather, export_only);
}

// LBM::Init (lbm.cpp:31-57) on the fluid cells: f = feq(rho, u), g =
// rho w T P3(u) (Calc_geq, lbm.cpp:636-653), shifted; aux = (rho - 1, u),
// aux2 = (0, F).  fields: [8][N] rho, u, T, F of the set-up.
__global__ void k_e3_init(float *__restrict__ A, float *__restrict__ GA, float4 *__restrict__ aux,
                          float4 *__restrict__ aux2, const int *__restrict__ rec_of, const float *__restrict__ fields,
                          const __grid_constant__ E3Params P) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= P.N || rec_of[c] == kSolid) return;
    const float rho = fields[c], ux = fields[P.N + c], uy = fields[2 * P.N + c], uz = fields[3 * P.N + c];
    const float T = fields[4 * P.N + c];
    const float usq = ux * ux + uy * uy + uz * uz;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float pm = p3m1(cu, usq);
        A[l * P.S + c] = wf(l) * ((rho - 1.0f) + rho * pm);
        GA[l * P.S + c] = wf(l) * ((rho * T - P.T_ref) + rho * T * pm);
    }
    aux[c] = make_float4(rho - 1.0f, ux, uy, uz);
    aux2[c] = make_float4(0.0f, fields[5 * P.N + c], fields[6 * P.N + c], fields[7 * P.N + c]);
}

// What MacroProp leaves on a wall cell (its f and g never change after
// Init): the set-up values before the first MacroProp, then the sums of
// its initial populations, with u = u_set + F / (2 rho) for the force of the
// previous MacroProp (the set-up one at MacroProp 1, the refreshed one
// later); q = sum g c = 0 (Init puts the walls' g at rest).
struct E3Wall {
    long long cell;
    double rho0, rhom, T0, Tm;
    double u[3][3];  // after 0, 1, >= 2 MacroProps
};

lbm_status fail3(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

}  // namespace

struct lbm_energy3d {
    E3Params P{};
    int nx = 0, ny = 0, nz = 0;
    float *f[2] = {nullptr, nullptr}, *g[2] = {nullptr, nullptr};
    float4 *aux = nullptr, *aux2 = nullptr;
    int *rec_of = nullptr;
    void *recbuf = nullptr;  // the records' field arrays
    E3Recs recs{};
    float *gold = nullptr, *tw = nullptr, *mom = nullptr, *fields = nullptr;
    float *scr = nullptr;  // the records' gathered f and g, [2 Q][records]
    uint32_t *status = nullptr;
    bool has_neu = false, inited = false;
    int cur = 0;
    long long steps = 0;
    cudaStream_t s = nullptr;
    cudaStream_t s2 = nullptr;  // the wall records, beside the bulk kernel (high priority)
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr, join = nullptr;
    // steps per captured graph (even, so that a replay ends on the buffer it
    // started from); 0: every step launched on its own
    int graph_steps = 0;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};  // by the starting buffer
    std::vector<void *> allocs;
    std::vector<E3Wall> walls;
};

namespace {

template <class Tp>
cudaError_t alloc3(lbm_energy3d *e, Tp **p, size_t bytes) {
    cudaError_t err = cudaMalloc((void **)p, bytes);
    if (err == cudaSuccess) e->allocs.push_back((void *)*p);
    else *p = nullptr;
    return err;
}

void free3(lbm_energy3d *e) {
    for (cudaGraphExec_t g : e->gexec)
        if (g) cudaGraphExecDestroy(g);
    for (void *p : e->allocs) cudaFree(p);
    if (e->s) cudaStreamDestroy(e->s);
    if (e->s2) cudaStreamDestroy(e->s2);
    if (e->fork) cudaEventDestroy(e->fork);
    if (e->join) cudaEventDestroy(e->join);
    for (cudaEvent_t v : e->ev)
        if (v) cudaEventDestroy(v);
    delete e;
}

int phase_of(long long steps) { return steps <= 1 ? 0 : (steps == 2 ? 1 : 2); }

// The wall records.  type/te/T/rho/u/F: the set-up arrays (ghost-inclusive).
// Replays the reference's push order (i outer, j, k inner) over the fluid
// cells to find, for each solid neighbour of a cell, the last Neumann write
// of its T before the cell (Determine_Twall_Neumann's write of the cell
// opposite the normal, lbm.cpp:1021-1027, and the write of each Neumann
// wall cell, lbm.cpp:284).
lbm_status build_records(const lbm_energy3d_setup &su, int NX, int NY, int NZ, double gbeta, double T_star,
                         bool buoy, const std::vector<double> &rho, const std::vector<double> &F,
                         std::vector<int> &rec_of, std::vector<E3Rec> &recs, std::vector<E3Wall> &walls) {
    const long long N = (long long)NX * NY * NZ;
    auto idx = [&](int i, int j, int k) { return (long long)i + (long long)NX * (j + (long long)NY * k); };
    auto nb = [&](long long c, int l) {
        const int i = (int)(c % NX), j = (int)((c / NX) % NY), k = (int)(c / ((long long)NX * NY));
        return idx((i + cx(l) + NX) % NX, (j + cy(l) + NY) % NY, (k + cz(l) + NZ) % NZ);
    };
    auto solid = [&](long long c) { return su.type[c] == kTypeS; };
    // A wall's g and f never change after Init, so MacroProp gives it the
    // same T and rho every step: the sums, in the reference's order and
    // rounding, of its initial g = rho w T_w (Calc_geq at rest, T_w the mean
    // set-up T of its solid neighbours, Determine_Wall_Temperature) and f =
    // rho w.  The rounding matters: Determine_Wall_Velocity counts the walls
    // with u != 0, and a wall whose exact T is T* moves at about 1e-21
    // (this file is compiled without floating-point contraction).
    std::vector<double> Twall(N, 0.0), rho_w(N, 1.0);
    for (long long c = 0; c < N; c++) {
        if (!solid(c)) continue;
        double s = 0.0;
        int num = 0;
        for (int l = 0; l < Q; l++) {
            const long long n = nb(c, l);
            if (solid(n)) {
                s += su.T[n];
                num++;
            }
        }
        if (!num) {
            Twall[c] = NAN;
            continue;
        }
        const double Tw = s / num;
        double Tm = 0.0, rm = 0.0;
        for (int l = 0; l < Q; l++) {
            Tm += rho[c] * wd(l) * Tw;
            rm += rho[c] * wd(l);
        }
        Twall[c] = Tm;
        rho_w[c] = rm;
    }
    // the walls' velocity at streaming 1 (set-up), 2 (after MacroProp 1)
    // and later (after MacroProp 2): u_set + F / (2 rho_w), F the force of
    // the previous MacroProp (the set-up one, then the refreshed one)
    auto wall_u = [&](long long w, int ph, double out[3]) {
        const double *u = su.u;
        for (int a = 0; a < 3; a++) {
            double v = u ? u[a * N + w] : 0.0;
            if (ph >= 1) {
                double Fa = F[a * N + w];
                if (ph == 2 && buoy && a == 1) Fa = gbeta * (Twall[w] - T_star);
                v += 0.5 * Fa / rho_w[w];
            }
            out[a] = v;
        }
    };
    walls.clear();
    for (long long c = 0; c < N; c++) {
        if (!solid(c)) continue;
        E3Wall W;
        W.cell = c;
        W.rho0 = rho[c];
        W.rhom = rho_w[c];
        W.T0 = su.T[c];
        W.Tm = Twall[c];
        for (int ph = 0; ph < 3; ph++) wall_u(c, ph, W.u[ph]);
        walls.push_back(W);
    }
    rec_of.assign(N, kSolid);
    recs.clear();
    std::vector<E3Slots> slots;
    for (long long c = 0; c < N; c++) {
        if (su.type[c] != kTypeF) continue;
        bool any = false;
        for (int l = 1; l < Q && !any; l++) any = solid(nb(c, l));
        if (!any) {
            const int i = (int)(c % NX), j = (int)((c / NX) % NY), k = (int)(c / ((long long)NX * NY));
            const bool face = i == 0 || i == NX - 1 || j == 0 || j == NY - 1 || k == 0 || k == NZ - 1;
            rec_of[c] = face ? kBulkWrap : kBulk;
            continue;
        }
        E3Rec R;
        memset(&R, 0, sizeof(R));
        R.cell = (int)c;
        R.i = (int)(c % NX);
        R.j = (int)((c / NX) % NY);
        R.k = (int)(c / ((long long)NX * NY));
        E3Slots L;
        for (int m = 0; m < kSlots; m++) {
            L.writer[m] = -1;
            L.own[m] = 255;
        }
        for (int ph = 0; ph < 3; ph++) {
            double s[3] = {0, 0, 0};
            int num = 0;
            for (int l = 0; l < Q; l++) {
                const long long w = nb(c, l);
                if (!solid(w)) continue;
                double uw[3];
                wall_u(w, ph, uw);
                if (uw[0] != 0 || uw[1] != 0 || uw[2] != 0) {
                    for (int a = 0; a < 3; a++) s[a] += uw[a];
                    num++;
                }
            }
            for (int a = 0; a < 3; a++) R.uw[ph][a] = (float)(num ? s[a] / num : 0.0);
        }
        for (int l = 0; l < Q; l++) {
            const long long w = nb(c, l);
            if (!solid(w)) continue;
            const int p = opp(l);
            R.bb |= 1u << p;
            const int te = su.type_energy[w];
            if (te == kTypeT) R.dir |= 1u << p;
            else if (te == kTypeQ) R.neu |= 1u << p;
            else R.adi |= 1u << p;
            if (!(std::isfinite(Twall[w])))
                return fail3(LBM_ERR_UNSUPPORTED, "energy3d_create: a wall cell next to fluid has no solid "
                                                  "neighbour (Determine_Wall_Temperature divides by zero)");
            L.cell[L.nsol] = w;
            L.tsol[0][L.nsol] = (float)su.T[w];
            L.tsol[1][L.nsol] = (float)Twall[w];
            L.nsol++;
        }
        rec_of[c] = (int)recs.size();
        recs.push_back(R);
        slots.push_back(L);
    }
    // the push order, replayed: last_writer[w] = record of the last
    // Neumann write of solid w so far
    std::vector<int> last_writer(N, -1);
    for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++)
            for (int k = 0; k < NZ; k++) {
                const long long c = idx(i, j, k);
                const int r = rec_of[c];
                if (r < 0) continue;
                const E3Rec &R = recs[r];
                E3Slots &L = slots[r];
                for (int m = 0; m < L.nsol; m++) L.writer[m] = last_writer[L.cell[m]];
                if (!R.neu) continue;
                // this cell's writes: at its first Neumann link the cell
                // opposite the normal (when the normal is a lattice
                // direction), at each Neumann link that link's wall cell
                double n[3] = {0, 0, 0};
                int np = 0;
                for (int l = 0; l < Q; l++)
                    if (solid(nb(c, l))) {
                        n[0] += cx(opp(l));
                        n[1] += cy(opp(l));
                        n[2] += cz(opp(l));
                        np++;
                    }
                for (int a = 0; a < 3; a++) n[a] /= np;
                long long wn = -1;
                for (int l = 0; l < Q; l++) {
                    const int o = opp(l);
                    if (cx(o) == n[0] && cy(o) == n[1] && cz(o) == n[2]) {
                        wn = nb(c, l);
                        break;
                    }
                }
                bool first = true;
                std::vector<long long> written;
                for (int l = 0; l < Q; l++) {
                    const long long w = nb(c, l);
                    if (!solid(w) || su.type_energy[w] != kTypeQ) continue;
                    const long long targets[2] = {first ? wn : -1, w};
                    first = false;
                    for (long long t : targets) {
                        if (t < 0) continue;
                        for (int s = 0; s < L.nsol; s++)
                            if (L.cell[s] == t && L.own[s] == 255) L.own[s] = (uint8_t)l;
                        written.push_back(t);
                    }
                }
                for (long long t : written) last_writer[t] = r;
            }
    // the compact form: static neighbours summed, dynamic ones listed
    for (size_t r = 0; r < recs.size(); r++) {
        E3Rec &R = recs[r];
        const E3Slots &L = slots[r];
        R.inv_nsol = 1.0f / (float)L.nsol;
        double s0 = 0.0, s1 = 0.0;
        for (int m = 0; m < L.nsol; m++) {
            if (L.writer[m] < 0 && L.own[m] == 255) {
                s0 += L.tsol[0][m];
                s1 += L.tsol[1][m];
                continue;
            }
            const int d = R.ndyn++;
            R.dwriter[d] = L.writer[m];
            R.down[d] = L.own[m];
            R.dt[0][d] = L.tsol[0][m];
            R.dt[1][d] = L.tsol[1][m];
        }
        R.ssum[0] = (float)s0;
        R.ssum[1] = (float)s1;
    }
    return LBM_OK;
}

#define CK3(expr)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) return fail3(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// A launch on stream s that may begin while the stream's previous kernel
// finishes (programmatic dependent launch, when pdl): the kernel waits for
// that grid's results with cudaGridDependencySynchronize.
template <class... K, class... A>
cudaError_t launch3(bool pdl, unsigned grid, unsigned block, cudaStream_t s, void (*kern)(K...), A &&...args) {
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3(grid);
    c.blockDim = dim3(block);
    c.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&c, kern, std::forward<A>(args)...);
}

// One step: the Neumann pre-pass and the wall records on the second stream,
// beside the bulk kernel (they write disjoint cells and read only the
// previous step's arrays); the next step waits for both.
cudaError_t enqueue3(lbm_energy3d *e, float *mom, int export_only) {
    const E3Params &P = e->P;
    const int gather = e->steps > 0 ? 1 : 0;
    const int phase = phase_of(e->steps);
    cudaError_t err = cudaSuccess;
    if (P.nrec) {
        err = cudaEventRecord(e->fork, e->s);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(e->s2, e->fork, 0);
        if (err != cudaSuccess) return err;
        // a warp a record where the records are a large share of the grid
        // (their chain is the step), else a thread a record (a warp each
        // would crowd the bulk kernel beside them)
        const bool wide = (long long)P.nrec * 8 >= P.N;
        // the record chain's later kernels start behind the earlier ones
        // where the chain is the step (the warp forms); on large grids their
        // early blocks would take slots from the bulk kernel beside them
        bool behind = false;
        if (gather && e->has_neu) {
            behind = true;
            if (wide) {
                const unsigned nb = (unsigned)(((long long)P.nrec * 32 + kWallBlock - 1) / kWallBlock);
                k_e3_walls<<<nb, kWallBlock, 0, e->s2>>>(e->g[e->cur], e->aux, e->recs, e->gold, e->tw, P, phase,
                                                    export_only ? 0 : 1);
            } else {
                const unsigned nb = (unsigned)((P.nrec + kRecBlock - 1) / kRecBlock);
                k_e3_walls_t<<<nb, kRecBlock, 0, e->s2>>>(e->g[e->cur], e->aux, e->recs, e->gold, e->tw, P, phase,
                                                     export_only ? 0 : 1);
            }
        }
        const unsigned rb = (unsigned)((P.nrec + kRecBlock - 1) / kRecBlock);
        if (wide) {
            if (gather) {
                const unsigned gb = (unsigned)(((long long)P.nrec * 32 + kWallBlock - 1) / kWallBlock);
                err = launch3(behind, gb, kWallBlock, e->s2, k_e3_rgather, (const float *)e->f[e->cur],
                              (const float *)e->g[e->cur], (const float4 *)e->aux, e->recs, (const float *)e->gold,
                              (const float *)e->tw, e->scr, P, phase);
                if (err != cudaSuccess) return err;
                behind = true;
            }
            err = launch3(behind, rb, kRecBlock, e->s2, k_e3_rcollide, (const float *)e->f[e->cur],
                          e->f[1 - e->cur], (const float *)e->g[e->cur], e->g[1 - e->cur], e->aux, e->aux2, e->recs,
                          e->gold, (const float *)e->scr, P, e->status, mom, gather, export_only);
        } else {
            err = launch3(false, rb, kRecBlock, e->s2, k_e3_rec, (const float *)e->f[e->cur], e->f[1 - e->cur],
                          (const float *)e->g[e->cur], e->g[1 - e->cur], e->aux, e->aux2, e->recs, e->gold,
                          (const float *)e->tw, P, e->status, mom, gather, phase, export_only);
        }
        if (err != cudaSuccess) return err;
        err = cudaEventRecord(e->join, e->s2);
        if (err != cudaSuccess) return err;
    }
    const unsigned blocks = (unsigned)((P.N + kBlock - 1) / kBlock);
    k_e3_bulk<<<blocks, kBlock, 0, e->s>>>(e->f[e->cur], e->f[1 - e->cur], e->g[e->cur], e->g[1 - e->cur], e->aux,
                                          e->aux2, e->rec_of, P, e->status, mom, gather, export_only);
    if (P.nrec) err = cudaStreamWaitEvent(e->s, e->join, 0);
    if (err != cudaSuccess) return err;
    return cudaGetLastError();
}

// From the third step on every step enqueues the same launches (gather on,
// phase 2) on alternating buffers: graph_steps of them are captured once per
// starting buffer, the second stream's records joining the capture through
// the fork and join events, and replayed as one launch.
cudaError_t replay3(lbm_energy3d *e) {
    cudaGraphExec_t &x = e->gexec[e->cur];
    if (!x) {
        const int cur0 = e->cur;
        const long long steps0 = e->steps;
        cudaError_t err = cudaStreamBeginCapture(e->s, cudaStreamCaptureModeThreadLocal);
        if (err != cudaSuccess) return err;
        for (int n = 0; n < e->graph_steps && err == cudaSuccess; n++) {
            err = enqueue3(e, nullptr, 0);
            e->cur = 1 - e->cur;
            e->steps++;
        }
        e->cur = cur0;
        e->steps = steps0;
        cudaGraph_t g = nullptr;
        const cudaError_t end = cudaStreamEndCapture(e->s, &g);
        if (err == cudaSuccess) err = end;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&x, g, 0);
        if (g) cudaGraphDestroy(g);
        if (err != cudaSuccess) {
            x = nullptr;
            return err;
        }
    }
    return cudaGraphLaunch(x, e->s);
}

}  // namespace

extern "C" lbm_status lbmgpu_energy3d_create(const lbm_energy3d_setup *su, lbm_energy3d **out) {
    if (!su || !out || !su->type || !su->type_energy || !su->T || su->nx < 1 || su->ny < 1 || su->nz < 1)
        return fail3(LBM_ERR_INVALID, "energy3d_create: bad arguments");
    if (!(su->tau > 0.5) || !(su->tau_g > 0.5) || !(su->cp > 0))
        return fail3(LBM_ERR_INVALID, "energy3d_create: needs tau > 0.5, tau_g > 0.5 and cp > 0");
    *out = nullptr;
    const int NX = su->nx + 2, NY = su->ny + 2, NZ = su->nz + 2;
    const long long N = (long long)NX * NY * NZ;
    if (N > (1LL << 30)) return fail3(LBM_ERR_INVALID, "energy3d_create: more than 2^30 cells");
    double Tsum = 0.0;
    long long nf = 0;
    for (long long c = 0; c < N; c++) {
        if (su->type[c] == kTypeF) {
            Tsum += su->T[c];
            nf++;
        } else if (su->type[c] != kTypeS) {
            return fail3(LBM_ERR_UNSUPPORTED, "energy3d_create: cell types other than TYPE_F and TYPE_S");
        }
    }
    if (!nf) return fail3(LBM_ERR_INVALID, "energy3d_create: no fluid cell");
    std::vector<double> rho(N, 1.0), F(3 * N, 0.0);
    if (su->rho)
        for (long long c = 0; c < N; c++) rho[c] = su->rho[c];
    if (su->F)
        for (long long c = 0; c < 3 * N; c++) F[c] = su->F[c];
    bool forced = su->g_beta != 0.0;
    for (long long c = 0; c < 3 * N && !forced; c++) forced = su->type[c % N] == kTypeF && F[c] != 0.0;
    std::vector<int> rec_of;
    std::vector<E3Rec> recs;
    std::vector<E3Wall> walls;
    const bool buoy = su->g_beta != 0.0;
    lbm_status st = build_records(*su, NX, NY, NZ, su->g_beta, su->T_star, buoy, rho, F, rec_of, recs, walls);
    if (st != LBM_OK) return st;

    lbm_energy3d *e = new lbm_energy3d();
    e->walls.swap(walls);
    // 0: ten steps a graph; odd counts round up to the next even one
    if (su->graph_steps >= 0) {
        const int gs = su->graph_steps ? std::min(su->graph_steps, 1000) : 10;
        e->graph_steps = gs + (gs & 1);
    }
    e->nx = su->nx;
    e->ny = su->ny;
    e->nz = su->nz;
    E3Params &P = e->P;
    P.NX = NX;
    P.NY = NY;
    P.NZ = NZ;
    P.N = N;
    P.S = ((N + 255) / 256) * 256;
    P.nrec = (int)recs.size();
    for (int l = 0; l < Q; l++) P.offs[l] = cx(l) + NX * (cy(l) + NY * cz(l));
    const double cs2 = 1.0 / 3.0, tg = su->tau_g;
    P.omega = (float)(1.0 / su->tau);
    P.inv_tau_g = (float)(1.0 / tg);
    P.tg_fac = (float)((tg - 0.5) / (cs2 * tg));
    P.inv_cp = (float)(1.0 / su->cp);
    P.two_nu = (float)(2.0 * cs2 * (su->tau - 0.5));
    P.s_fac = (float)(-1.0 / (2.0 * su->tau * cs2));
    P.T_ref = (float)(Tsum / nf);
    P.gbeta = (float)su->g_beta;
    P.T_star = (float)su->T_star;
    P.buoy = buoy ? 1 : 0;
    P.forced = forced ? 1 : 0;
    for (const E3Rec &R : recs) e->has_neu = e->has_neu || R.neu != 0;
    auto bail = [&](lbm_status s) {
        free3(e);
        return s;
    };
#define CKE(expr)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return bail(fail3(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)));        \
    } while (0)
    CKE(cudaStreamCreateWithFlags(&e->s, cudaStreamNonBlocking));
    {
        int lo = 0, hi = 0;
        CKE(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        CKE(cudaStreamCreateWithPriority(&e->s2, cudaStreamNonBlocking, hi));
    }
    for (int i = 0; i < 2; i++) CKE(cudaEventCreate(&e->ev[i]));
    CKE(cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming));
    CKE(cudaEventCreateWithFlags(&e->join, cudaEventDisableTiming));
    for (int i = 0; i < 2; i++) {
        CKE(alloc3(e, &e->f[i], (size_t)Q * P.S * sizeof(float)));
        CKE(alloc3(e, &e->g[i], (size_t)Q * P.S * sizeof(float)));
    }
    CKE(alloc3(e, &e->aux, (size_t)P.S * sizeof(float4)));
    CKE(alloc3(e, &e->aux2, (size_t)P.S * sizeof(float4)));
    CKE(alloc3(e, &e->rec_of, (size_t)N * sizeof(int)));
    // the records, one array per field, each at a 256-byte boundary
    const size_t nr = std::max<size_t>(1, recs.size());
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) / 256 * 256;
        return at;
    };
    const size_t o_cell = take(4 * nr), o_ci = take(4 * nr), o_cj = take(4 * nr), o_ck = take(4 * nr);
    const size_t o_bb = take(4 * nr), o_dir = take(4 * nr), o_neu = take(4 * nr), o_ndyn = take(4 * nr);
    const size_t o_inv = take(4 * nr), o_ssum = take(8 * nr), o_uw = take(36 * nr);
    const size_t o_dw = take(4 * kSlots * nr), o_dt = take(8 * kSlots * nr), o_down = take(kSlots * nr);
    std::vector<uint8_t> hb(off, 0);
    auto put = [&](size_t at, size_t idx, const void *v, size_t sz) { memcpy(hb.data() + at + idx * sz, v, sz); };
    for (size_t r = 0; r < recs.size(); r++) {
        const E3Rec &R = recs[r];
        put(o_cell, r, &R.cell, 4);
        put(o_ci, r, &R.i, 4);
        put(o_cj, r, &R.j, 4);
        put(o_ck, r, &R.k, 4);
        put(o_bb, r, &R.bb, 4);
        put(o_dir, r, &R.dir, 4);
        put(o_neu, r, &R.neu, 4);
        put(o_ndyn, r, &R.ndyn, 4);
        put(o_inv, r, &R.inv_nsol, 4);
        for (int ph = 0; ph < 2; ph++) put(o_ssum, ph * nr + r, &R.ssum[ph], 4);
        for (int ph = 0; ph < 3; ph++)
            for (int a = 0; a < 3; a++) put(o_uw, (3 * ph + a) * nr + r, &R.uw[ph][a], 4);
        for (int m = 0; m < kSlots; m++) {
            put(o_dw, m * nr + r, &R.dwriter[m], 4);
            put(o_down, m * nr + r, &R.down[m], 1);
            for (int ph = 0; ph < 2; ph++) put(o_dt, (ph * kSlots + m) * nr + r, &R.dt[ph][m], 4);
        }
    }
    CKE(alloc3(e, &e->recbuf, off));
    CKE(cudaMemcpy(e->recbuf, hb.data(), off, cudaMemcpyHostToDevice));
    {
        const uint8_t *b = (const uint8_t *)e->recbuf;
        E3Recs &D = e->recs;
        D.cell = (const int *)(b + o_cell);
        D.ci = (const int *)(b + o_ci);
        D.cj = (const int *)(b + o_cj);
        D.ck = (const int *)(b + o_ck);
        D.bb = (const uint32_t *)(b + o_bb);
        D.dir = (const uint32_t *)(b + o_dir);
        D.neu = (const uint32_t *)(b + o_neu);
        D.ndyn = (const int *)(b + o_ndyn);
        D.inv_nsol = (const float *)(b + o_inv);
        D.ssum = (const float *)(b + o_ssum);
        D.uw = (const float *)(b + o_uw);
        D.dwriter = (const int *)(b + o_dw);
        D.dt = (const float *)(b + o_dt);
        D.down = (const uint8_t *)(b + o_down);
    }
    CKE(alloc3(e, &e->gold, (size_t)Q * std::max(1, P.nrec) * sizeof(float)));
    CKE(alloc3(e, &e->tw, (size_t)std::max(1, P.nrec) * sizeof(float)));
    CKE(alloc3(e, &e->scr, (size_t)2 * Q * std::max(1, P.nrec) * sizeof(float)));
    CKE(alloc3(e, &e->mom, (size_t)8 * N * sizeof(float)));
    CKE(alloc3(e, &e->fields, (size_t)8 * N * sizeof(float)));
    CKE(alloc3(e, &e->status, sizeof(uint32_t)));
    CKE(cudaMemcpy(e->rec_of, rec_of.data(), (size_t)N * sizeof(int), cudaMemcpyHostToDevice));

    std::vector<float> fl((size_t)8 * N);
    for (long long c = 0; c < N; c++) {
        fl[c] = (float)rho[c];
        for (int a = 0; a < 3; a++) fl[(1 + a) * N + c] = (float)(su->u ? su->u[a * N + c] : 0.0);
        fl[4 * N + c] = (float)su->T[c];
        for (int a = 0; a < 3; a++) fl[(5 + a) * N + c] = (float)F[a * N + c];
    }
    CKE(cudaMemcpy(e->fields, fl.data(), fl.size() * sizeof(float), cudaMemcpyHostToDevice));
#undef CKE
    *out = e;
    return lbmgpu_energy3d_init(e);
}

extern "C" lbm_status lbmgpu_energy3d_init(lbm_energy3d *e) {
    if (!e) return fail3(LBM_ERR_INVALID, "energy3d_init: null handle");
    const E3Params &P = e->P;
    CK3(cudaMemsetAsync(e->status, 0, sizeof(uint32_t), e->s));
    // NaN on the solid cells of the exported moments
    CK3(cudaMemsetAsync(e->mom, 0xff, (size_t)8 * P.N * sizeof(float), e->s));
    for (int i = 0; i < 2; i++) {
        CK3(cudaMemsetAsync(e->f[i], 0, (size_t)Q * P.S * sizeof(float), e->s));
        CK3(cudaMemsetAsync(e->g[i], 0, (size_t)Q * P.S * sizeof(float), e->s));
    }
    const unsigned blocks = (unsigned)((P.N + kBlock - 1) / kBlock);
    k_e3_init<<<blocks, kBlock, 0, e->s>>>(e->f[0], e->g[0], e->aux, e->aux2, e->rec_of, e->fields, P);
    CK3(cudaGetLastError());
    CK3(cudaStreamSynchronize(e->s));
    e->cur = 0;
    e->steps = 0;
    e->inited = true;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_energy3d_step(lbm_energy3d *e, int nsteps) {
    if (!e) return fail3(LBM_ERR_INVALID, "energy3d_step: null handle");
    if (!e->inited) return fail3(LBM_ERR_STATE, "energy3d_step: not initialised");
    if (nsteps < 0) return fail3(LBM_ERR_INVALID, "energy3d_step: negative count");
    for (int n = 0; n < nsteps;) {
        if (e->graph_steps > 0 && e->steps >= 3 && nsteps - n >= e->graph_steps) {
            CK3(replay3(e));
            e->steps += e->graph_steps;
            n += e->graph_steps;
            continue;
        }
        CK3(enqueue3(e, nullptr, 0));
        e->cur = 1 - e->cur;
        e->steps++;
        n++;
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_energy3d_step_timed(lbm_energy3d *e, int nsteps, double *ms) {
    if (!e || !ms) return fail3(LBM_ERR_INVALID, "energy3d_step_timed: bad arguments");
    CK3(cudaEventRecord(e->ev[0], e->s));
    lbm_status st = lbmgpu_energy3d_step(e, nsteps);
    if (st != LBM_OK) return st;
    CK3(cudaEventRecord(e->ev[1], e->s));
    CK3(cudaEventSynchronize(e->ev[1]));
    float t = 0.0f;
    CK3(cudaEventElapsedTime(&t, e->ev[0], e->ev[1]));
    *ms = t;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_energy3d_download(lbm_energy3d *e, int field, double *host) {
    if (!e || !host || field < LBM_FIELD_RHO || field > LBM_FIELD_QZ)
        return fail3(LBM_ERR_INVALID, "energy3d_download: bad arguments");
    if (!e->inited) return fail3(LBM_ERR_STATE, "energy3d_download: not initialised");
    // a gather-only pass over the current state (no collision, no store)
    CK3(enqueue3(e, e->mom, 1));
    const long long N = e->P.N;
    std::vector<float> buf(N);
    CK3(cudaMemcpyAsync(buf.data(), e->mom + (long long)field * N, N * sizeof(float), cudaMemcpyDeviceToHost, e->s));
    CK3(cudaStreamSynchronize(e->s));
    for (long long c = 0; c < N; c++) host[c] = buf[c];
    const int ph = e->steps < 2 ? (int)e->steps : 2;
    for (const E3Wall &W : e->walls) {
        double v = 0.0;
        switch (field) {
        case LBM_FIELD_RHO: v = e->steps ? W.rhom : W.rho0; break;
        case LBM_FIELD_UX: v = W.u[ph][0]; break;
        case LBM_FIELD_UY: v = W.u[ph][1]; break;
        case LBM_FIELD_UZ: v = W.u[ph][2]; break;
        case LBM_FIELD_T: v = e->steps ? W.Tm : W.T0; break;
        default: v = 0.0; break;
        }
        host[W.cell] = v;
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_energy3d_status(lbm_energy3d *e, uint32_t *flags) {
    if (!e || !flags) return fail3(LBM_ERR_INVALID, "energy3d_status: bad arguments");
    CK3(cudaMemcpyAsync(flags, e->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, e->s));
    CK3(cudaStreamSynchronize(e->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_energy3d_destroy(lbm_energy3d *e) {
    if (!e) return LBM_OK;
    if (e->s) cudaStreamSynchronize(e->s);
    free3(e);
    return LBM_OK;
}
