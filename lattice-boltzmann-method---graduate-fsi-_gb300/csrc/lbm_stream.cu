// lbm_stream.cu -- fused pull-scheme collide-stream kernels (D3Q19 + D3Q7).
//
// One launch of k_step advances every interior cell by one reference
// iteration in the fused order
//     gather (= LBM::Streaming of the previous step, lbm.cpp:182-296)
//  -> moments (= LBM::MacroProp, lbm.cpp:668-679)
//  -> BGK + Guo collision (= LBM::Collision / ConvLBM, lbm.cpp:60-119)
// reading populations from buffer A and writing post-collision populations
// to buffer B (A/B ping-pong).  Halfway bounce-back with the per-cell wall
// velocity of Determine_Wall_Velocity (lbm.cpp:941-962), inlet/outlet
// equilibrium ghosts and zero-gradient outlets are folded into the gather
// through a per-boundary-class table (see ClassEntry).  Cells inside the IBM
// band store their pre-collision populations and unforced moments instead;
// k_band_collide finishes them once the IBM forcing is known.
#include "lbm_device.cuh"
#include "lbm_internal.h"

namespace lbmk {

template <class T>
__device__ __forceinline__ void gather_flow(const T *__restrict__ A, float f[Q], int x, int y, int z,
                                            long long cell, int raw_cls, bool valid, bool bwarp, int gather,
                                            const StepParams &P) {
    const long long N = P.N;
    if (!gather) {
#pragma unroll
        for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(A + l * N + cell) : 0.0f;
        return;
    }
    if (!bwarp) {
#pragma unroll
        for (int l = 0; l < Q; l++) {
            const long long off = (long long)cx(l) + (long long)P.nx * ((long long)cy(l) + (long long)P.ny * cz(l));
            f[l] = valid ? St<T>::ld(A + l * N + cell - off) : 0.0f;
        }
        return;
    }
    const int pm = ((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0) | ((P.periodic & 4) ? 48 : 0);
    const ClassEntry &ce = P.cls[raw_cls & ~pm];
#pragma unroll
    for (int l = 0; l < Q; l++) {
        float v = 0.0f;
        if (valid) {
            if ((ce.bb >> l) & 1u) {
                v = St<T>::ld(A + opp(l) * N + cell) + ce.val[l];
            } else if ((ce.eq >> l) & 1u) {
                v = ce.val[l];
            } else {
                int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
                // periodic axes wrap; a zero-gradient link then clamps the
                // remaining ghost coordinates onto the interior
                if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
                if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
                if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
                if ((ce.zg >> l) & 1u) {
                    sx = min(max(sx, 0), P.nx - 1);
                    sy = min(max(sy, 0), P.ny - 1);
                    sz = min(max(sz, 0), P.nz - 1);
                }
                v = St<T>::ld(A + l * N + sx + (long long)P.nx * (sy + (long long)P.ny * sz));
            }
        }
        f[l] = v;
    }
}

template <class T>
__device__ __forceinline__ void gather_heat(const T *__restrict__ G, float g[QT], int x, int y, int z,
                                            long long cell, int raw_cls, bool valid, bool bwarp, int gather,
                                            const StepParams &P) {
    const long long N = P.N;
    if (!gather) {
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = valid ? St<T>::ld(G + l * N + cell) : 0.0f;
        return;
    }
    if (!bwarp) {
#pragma unroll
        for (int l = 0; l < QT; l++) {
            const long long off = (long long)cx(l) + (long long)P.nx * ((long long)cy(l) + (long long)P.ny * cz(l));
            g[l] = valid ? St<T>::ld(G + l * N + cell - off) : 0.0f;
        }
        return;
    }
    const int pm = ((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0) | ((P.periodic & 4) ? 48 : 0);
    const ClassEntry &ce = P.cls[raw_cls & ~pm];
#pragma unroll
    for (int l = 0; l < QT; l++) {
        float v = 0.0f;
        if (valid) {
            if ((ce.bb >> l) & 1u) {
                float own = St<T>::ld(G + opp(l) * N + cell);
                v = ((ce.tdir >> l) & 1u) ? (-own + ce.tval[l]) : own;
            } else if ((ce.eq >> l) & 1u) {
                v = ce.tval[l];
            } else {
                int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
                // periodic axes wrap; a zero-gradient link then clamps the
                // remaining ghost coordinates onto the interior
                if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
                if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
                if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
                if ((ce.zg >> l) & 1u) {
                    sx = min(max(sx, 0), P.nx - 1);
                    sy = min(max(sy, 0), P.ny - 1);
                    sz = min(max(sz, 0), P.nz - 1);
                }
                v = St<T>::ld(G + l * N + sx + (long long)P.nx * (sy + (long long)P.ny * sz));
            }
        }
        g[l] = v;
    }
}

// BGK + Guo collision on shifted populations (f~ = f - w), FP32:
//   f~* = (1 - omega) f~ + omega (feq - w) + S,
//   feq - w = w (drho + rho P3(u)) with the third-order P3 of Calc_feq
//   (lbm.cpp:628-633), S = (1 - omega/2) w (3 c.F + 9 (c.F)(c.u) - 3 F.u)
//   (lbm.cpp:101-102).
__device__ __forceinline__ void collide_flow(float f[Q], float drho, float ux, float uy, float uz, float Fx,
                                             float Fy, float Fz, bool forced, float omega) {
    const float rho = 1.0f + drho;
    const float usq = ux * ux + uy * uy + uz * uz;
    const float c1 = 1.0f - omega;
    const float gs = 1.0f - 0.5f * omega;
    const float Fu = Fx * ux + Fy * uy + Fz * uz;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float p3 = cu * (3.0f + 4.5f * cu + 4.5f * cu * cu - 4.5f * usq) - 1.5f * usq;
        float out = c1 * f[l] + omega * wf(l) * (drho + rho * p3);
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
template <class T, bool THERMAL>
__global__ void __launch_bounds__(256) k_step(const T *__restrict__ A, T *__restrict__ B, const T *__restrict__ GA,
                                              T *__restrict__ GB, const __grid_constant__ StepParams P,
                                              DevState *__restrict__ ds, float *__restrict__ mom,
                                              float *__restrict__ band, int gather, int export_only) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool valid = (x < P.nx) && (y < P.ny);
    const long long N = P.N;
    const long long cell = valid ? (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z) : 0;
    const int raw = valid ? ((x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                             (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0))
                          : 0;
    const bool bwarp = __any_sync(0xffffffffu, raw != 0);

    float f[Q];
    gather_flow<T>(A, f, x, y, z, cell, raw, valid, bwarp, gather, P);
    float drho = 0.0f, jx = 0.0f, jy = 0.0f, jz = 0.0f;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        drho += f[l];
        jx += cx(l) * f[l];
        jy += cy(l) * f[l];
        jz += cz(l) * f[l];
    }
    float g[QT];
    float Tc = 0.0f;
    float Fx = P.body[0], Fy = P.body[1], Fz = P.body[2];
    if (THERMAL) {
        gather_heat<T>(GA, g, x, y, z, cell, raw, valid, bwarp, gather, P);
#pragma unroll
        for (int l = 0; l < QT; l++) Tc += g[l];
        Fx += P.gbeta[0] * (Tc - P.T0);
        Fy += P.gbeta[1] * (Tc - P.T0);
        Fz += P.gbeta[2] * (Tc - P.T0);
    }
    const float rho = 1.0f + drho;
    const float inv = 1.0f / rho;
    // Before the first streaming the reference collides with the velocity
    // stored at set-up (LBM::Init, lbm.cpp:31-57), i.e. without the F/2 shift
    // that MacroProp applies afterwards (lbm.cpp:677-679).
    const float hf = gather ? 0.5f : 0.0f;
    const float ux = (jx + hf * Fx) * inv;
    const float uy = (jy + hf * Fy) * inv;
    const float uz = (jz + hf * Fz) * inv;
    if (valid && !(rho > 0.0f && rho < 100.0f)) atomicOr(&ds->status, ST_RHO_RANGE);
    if (mom != nullptr && valid) {
        mom[cell] = rho;
        mom[N + cell] = ux;
        mom[2 * N + cell] = uy;
        mom[3 * N + cell] = uz;
        if (THERMAL) mom[4 * N + cell] = Tc;
    }
    if (export_only || !valid) return;

    if (P.band_on) {
        const int bx = x - ds->band_o[0], by = y - ds->band_o[1], bz = z - ds->band_o[2];
        if ((unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz) {
            const long long nb = P.nb;
            const long long b = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
#pragma unroll
            for (int l = 0; l < Q; l++) St<T>::st(B + l * N + cell, f[l]);
            if (THERMAL) {
#pragma unroll
                for (int l = 0; l < QT; l++) St<T>::st(GB + l * N + cell, g[l]);
            }
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
            return;
        }
    }
    collide_flow(f, drho, ux, uy, uz, Fx, Fy, Fz, P.forced != 0, P.omega);
#pragma unroll
    for (int l = 0; l < Q; l++) St<T>::st(B + l * N + cell, f[l]);
    if (THERMAL) {
        collide_heat(g, Tc, ux, uy, uz, 0.0f, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * N + cell, g[l]);
    }
}

// Collision of the IBM band cells, after the forcing iterations: rho and the
// unforced velocity from k_step, the accumulated IBM force Ft (band[7..9])
// and heat source (band[11]).  u = u_unf + Ft / (2 rho) and F = Fb + sign Ft
// (sign = -1 reproduces lbm.cpp:1347-1352); T = T_unf + Qt / 2.
template <class T, bool THERMAL>
__global__ void __launch_bounds__(256) k_band_collide(T *__restrict__ B, T *__restrict__ GB,
                                                      const __grid_constant__ StepParams P,
                                                      const DevState *__restrict__ ds,
                                                      const float *__restrict__ band, float fsign) {
    const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (b >= P.nb) return;
    const int bx = (int)(b % P.bsx);
    const int by = (int)((b / P.bsx) % P.bsy);
    const int bz = (int)(b / ((long long)P.bsx * P.bsy));
    const int x = bx + ds->band_o[0], y = by + ds->band_o[1], z = bz + ds->band_o[2];
    if (x < 0 || y < 0 || z < 0 || x >= P.nx || y >= P.ny || z >= P.nz) return;
    const long long N = P.N, nb = P.nb;
    const long long cell = x + (long long)P.nx * (y + (long long)P.ny * z);
    float f[Q];
#pragma unroll
    for (int l = 0; l < Q; l++) f[l] = St<T>::ld(B + l * N + cell);
    const float drho = band[b];
    const float rho = 1.0f + drho;
    const float ftx = band[7 * nb + b], fty = band[8 * nb + b], ftz = band[9 * nb + b];
    const float ux = band[nb + b] + 0.5f * ftx / rho;
    const float uy = band[2 * nb + b] + 0.5f * fty / rho;
    const float uz = band[3 * nb + b] + 0.5f * ftz / rho;
    const float Fx = band[4 * nb + b] + fsign * ftx;
    const float Fy = band[5 * nb + b] + fsign * fty;
    const float Fz = band[6 * nb + b] + fsign * ftz;
    collide_flow(f, drho, ux, uy, uz, Fx, Fy, Fz, true, P.omega);
#pragma unroll
    for (int l = 0; l < Q; l++) St<T>::st(B + l * N + cell, f[l]);
    if (THERMAL) {
        float g[QT];
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = St<T>::ld(GB + l * N + cell);
        const float Qt = band[11 * nb + b];
        const float Tc = band[10 * nb + b] + 0.5f * Qt;
        collide_heat(g, Tc, ux, uy, uz, Qt, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * N + cell, g[l]);
    }
}

// Initial populations (LBM::Init, lbm.cpp:31-57): f = feq3(rho, u) stored
// shifted, g = geq(T, u); from uniform values or per-cell host fields.
template <class T, bool THERMAL>
__global__ void k_init(T *__restrict__ A, T *__restrict__ GA, long long N, const float *__restrict__ fields,
                       float rho0, float ux0, float uy0, float uz0, float T0) {
    const long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (c >= N) return;
    float drho = rho0 - 1.0f, ux = ux0, uy = uy0, uz = uz0, Tc = T0;
    if (fields != nullptr) {
        drho = fields[c] - 1.0f;
        ux = fields[N + c];
        uy = fields[2 * N + c];
        uz = fields[3 * N + c];
        if (THERMAL) Tc = fields[4 * N + c];
    }
    const float rho = 1.0f + drho;
    const float usq = ux * ux + uy * uy + uz * uz;
#pragma unroll
    for (int l = 0; l < Q; l++) {
        const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
        const float p3 = cu * (3.0f + 4.5f * cu + 4.5f * cu * cu - 4.5f * usq) - 1.5f * usq;
        St<T>::st(A + l * N + c, wf(l) * (drho + rho * p3));
    }
    if (THERMAL) {
#pragma unroll
        for (int l = 0; l < QT; l++) {
            const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
            St<T>::st(GA + l * N + c, wtf(l) * Tc * (1.0f + 4.0f * cu));
        }
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
template <class T>
static cudaError_t launch_step_t(const LaunchArgs &a) {
    dim3 blk(a.tx, a.ty, 1);
    dim3 grd((a.P->nx + a.tx - 1) / a.tx, (a.P->ny + a.ty - 1) / a.ty, a.P->nz);
    if (a.thermal)
        k_step<T, true><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, (const T *)a.GA, (T *)a.GB, *a.P, a.ds,
                                                   a.mom, a.band, a.gather, a.export_only);
    else
        k_step<T, false><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, nullptr, nullptr, *a.P, a.ds, a.mom,
                                                    a.band, a.gather, a.export_only);
    return cudaGetLastError();
}

cudaError_t launch_step(int storage, const LaunchArgs &a) {
    switch (storage) {
    case 0: return launch_step_t<float>(a);
    case 1: return launch_step_t<__half>(a);
    case 2: return launch_step_t<__nv_bfloat16>(a);
    }
    return cudaErrorInvalidValue;
}

template <class T>
static cudaError_t launch_band_t(const LaunchArgs &a, float fsign) {
    int threads = 256;
    long long blocks = (a.P->nb + threads - 1) / threads;
    if (a.thermal)
        k_band_collide<T, true><<<(unsigned)blocks, threads, 0, a.stream>>>((T *)a.B, (T *)a.GB, *a.P, a.ds, a.band,
                                                                            fsign);
    else
        k_band_collide<T, false><<<(unsigned)blocks, threads, 0, a.stream>>>((T *)a.B, nullptr, *a.P, a.ds, a.band,
                                                                             fsign);
    return cudaGetLastError();
}

cudaError_t launch_band_collide(int storage, const LaunchArgs &a, float fsign) {
    switch (storage) {
    case 0: return launch_band_t<float>(a, fsign);
    case 1: return launch_band_t<__half>(a, fsign);
    case 2: return launch_band_t<__nv_bfloat16>(a, fsign);
    }
    return cudaErrorInvalidValue;
}

template <class T>
static cudaError_t launch_init_t(void *A, void *GA, long long N, const float *fields, const float init[5], bool thermal,
                                 cudaStream_t s) {
    int threads = 256;
    long long blocks = (N + threads - 1) / threads;
    if (thermal)
        k_init<T, true><<<(unsigned)blocks, threads, 0, s>>>((T *)A, (T *)GA, N, fields, init[0], init[1], init[2],
                                                             init[3], init[4]);
    else
        k_init<T, false><<<(unsigned)blocks, threads, 0, s>>>((T *)A, nullptr, N, fields, init[0], init[1], init[2],
                                                              init[3], init[4]);
    return cudaGetLastError();
}

cudaError_t launch_init(int storage, void *A, void *GA, long long N, const float *fields, const float init[5],
                        bool thermal, cudaStream_t s) {
    switch (storage) {
    case 0: return launch_init_t<float>(A, GA, N, fields, init, thermal, s);
    case 1: return launch_init_t<__half>(A, GA, N, fields, init, thermal, s);
    case 2: return launch_init_t<__nv_bfloat16>(A, GA, N, fields, init, thermal, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lbmk
