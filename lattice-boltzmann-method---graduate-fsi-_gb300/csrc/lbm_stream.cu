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
#include "lbm_internal.h"
#include "lbm_step.cuh"

namespace lbmk {

// Fused step, direct global loads (any row length).  gather = 0 on the first
// step (A then holds the initial pre-collision populations in place);
// export_only = 1 computes and writes the moments of the gathered state
// without colliding or storing.
template <class T, bool THERMAL, bool FORCED, bool SOLID>
__global__ void __launch_bounds__(256, (THERMAL || SOLID) ? 4 : (FORCED ? 5 : 6))
    k_step(const T *__restrict__ A, T *__restrict__ B, const T *__restrict__ GA, T *__restrict__ GB,
           const __grid_constant__ StepParams P, DevState *__restrict__ ds, float *__restrict__ mom,
           float *__restrict__ band, int gather, int export_only, int region) {
    // region 0: every cell; 1: all but the near box; 2: only the near box
    // (the grid spans it).  The near box [nlo, nhi) holds the IBM band grown
    // by the one-cell pull stencil, rounded out to whole tiles.
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    int z = blockIdx.z;
    bool valid;
    if (region == 2) {
        x += P.nlo[0];
        y += P.nlo[1];
        z += P.nlo[2];
        valid = x < P.nhi[0] && y < P.nhi[1] && z < P.nhi[2];
    } else {
        valid = (x < P.nx) && (y < P.ny);
        if (region == 1 && x >= P.nlo[0] && x < P.nhi[0] && y >= P.nlo[1] && y < P.nhi[1] && z >= P.nlo[2] &&
            z < P.nhi[2])
            valid = false;
    }
    const long long cell = valid ? (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z) : 0;
    const int raw = valid ? ((x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                             (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0))
                          : 0;
    float f[Q], g[QT];
    if (SOLID) {
        // warps near an interior solid take the solid-aware pull
        const bool swarp = __any_sync(0xffffffffu, valid && mask_bit(P.nearw, cell));
        float mea[3] = {0.0f, 0.0f, 0.0f};
        if (swarp) {
            const bool sc = valid && mask_bit(P.solid, cell);
            gather_solid<T, THERMAL>(A, GA, f, g, x, y, z, cell, raw, valid, sc, gather, P, mea);
            finish_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, gather, export_only, B, GB, P, ds, mom,
                                            band, region != 1, sc);
        } else {
            const bool bwarp = __any_sync(0xffffffffu, (P.xface ? (raw & ~3) : raw) != 0);
            gather_flow<T>(A, f, x, y, z, cell, raw, valid, bwarp, gather, P);
            if (THERMAL) gather_heat<T>(GA, g, x, y, z, cell, raw, valid, bwarp, gather, P);
            finish_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, gather, export_only, B, GB, P, ds, mom,
                                            band, region != 1);
        }
        // per-block momentum exchange, summed in a fixed order
        if (P.mea != nullptr && gather && region == 0 && __syncthreads_or(swarp ? 1 : 0)) {
            __shared__ float part[8][3];
            const int t = threadIdx.x + blockDim.x * threadIdx.y, lane = t & 31, w = t >> 5;
#pragma unroll
            for (int k = 0; k < 3; k++) {
                float v = mea[k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (lane == 0) part[w][k] = v;
            }
            __syncthreads();
            if (t == 0) {
                const int nw = (blockDim.x * blockDim.y + 31) >> 5;
                const long long b = blockIdx.x + (long long)gridDim.x * (blockIdx.y + (long long)gridDim.y * blockIdx.z);
                for (int k = 0; k < 3; k++) {
                    float v = 0.0f;
                    for (int i = 0; i < nw; i++) v += part[i][k];
                    P.mea[3 * b + k] = v;
                }
            }
        }
        return;
    }
    // With xface, x-face lanes of rows off the y/z faces stay on the plain
    // path and fix their x-crossing links themselves (gather_flow); idle
    // lanes take whichever path their warp takes.
    const int rawrow = P.xface ? (raw & ~3) : raw;
    const bool bwarp = __any_sync(0xffffffffu, rawrow != 0);
    gather_flow<T>(A, f, x, y, z, cell, raw, valid, bwarp, gather, P);
    if (THERMAL) gather_heat<T>(GA, g, x, y, z, cell, raw, valid, bwarp, gather, P);
    finish_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, gather, export_only, B, GB, P, ds, mom, band,
                                    region != 1);
}

// Collision of the IBM band cells after the forcing iterations
// (band_collide_cell).  64-thread blocks of at most 64 registers: they fit
// beside the far-region collide-stream blocks (which leave 4096 registers
// per SM) when overlapped.
template <class T, bool THERMAL>
__global__ void __launch_bounds__(64, 16) k_band_collide(T *__restrict__ B, T *__restrict__ GB,
                                                      const __grid_constant__ StepParams P,
                                                      const DevState *__restrict__ ds,
                                                      float *__restrict__ band, float fsign) {
    // the last spreading may still be running (programmatic dependent launch)
    cudaGridDependencySynchronize();
    const long long b = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (b >= P.nb) return;
    band_collide_cell<T, THERMAL>(B, GB, P, ds, band, fsign, b);
}

// Initial populations (LBM::Init, lbm.cpp:31-57): f = feq3(rho, u) stored
// shifted, g = geq(T, u); from uniform values or per-cell host fields.
template <class T, bool THERMAL>
__global__ void k_init(T *__restrict__ A, T *__restrict__ GA, T *__restrict__ A2, T *__restrict__ GA2, long long N,
                       long long S, const float *__restrict__ fields, float rho0, float ux0, float uy0, float uz0,
                       float T0) {
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
        const float v = wf(l) * (drho + rho * p3);
        St<T>::st(A + l * S + c, v);
        if (A2) St<T>::st(A2 + l * S + c, v);
    }
    if (THERMAL) {
#pragma unroll
        for (int l = 0; l < QT; l++) {
            const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
            const float v = wtf(l) * Tc * (1.0f + 4.0f * cu);
            St<T>::st(GA + l * S + c, v);
            if (GA2) St<T>::st(GA2 + l * S + c, v);
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
    const bool forced = a.P->forced != 0;
    if (a.region == 2) {
        // the near box is a few tens of cells wide: 32 x 8 blocks keep few lanes idle
        blk = dim3(32, 8, 1);
        grd = dim3((a.P->nhi[0] - a.P->nlo[0] + 31) / 32, (a.P->nhi[1] - a.P->nlo[1] + 7) / 8,
                   a.P->nhi[2] - a.P->nlo[2]);
    }
    const T *A = (const T *)a.A, *GA = (const T *)a.GA;
    T *B = (T *)a.B, *GB = (T *)a.GB;
    if (a.P->solid != nullptr) {
        if (a.thermal)
            k_step<T, true, true, true><<<grd, blk, 0, a.stream>>>(A, B, GA, GB, *a.P, a.ds, a.mom, a.band, a.gather,
                                                                  a.export_only, a.region);
        else if (forced)
            k_step<T, false, true, true><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, *a.P, a.ds, a.mom, a.band,
                                                                   a.gather, a.export_only, a.region);
        else
            k_step<T, false, false, true><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, *a.P, a.ds, a.mom,
                                                                    a.band, a.gather, a.export_only, a.region);
        return cudaGetLastError();
    }
    if (a.thermal)
        k_step<T, true, true, false><<<grd, blk, 0, a.stream>>>(A, B, GA, GB, *a.P, a.ds, a.mom, a.band, a.gather,
                                                               a.export_only, a.region);
    else if (forced)
        k_step<T, false, true, false><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, *a.P, a.ds, a.mom, a.band,
                                                                a.gather, a.export_only, a.region);
    else
        k_step<T, false, false, false><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, *a.P, a.ds, a.mom, a.band,
                                                                 a.gather, a.export_only, a.region);
    return cudaGetLastError();
}

cudaError_t launch_step(int storage, const LaunchArgs &a) {
    if (a.vcells > 1 && a.gather && !a.export_only && a.mom == nullptr && a.region != 2)
        return launch_step_vec(storage, a);
    switch (storage) {
    case 0: return launch_step_t<float>(a);
    case 1: return launch_step_t<__half>(a);
    case 2: return launch_step_t<__nv_bfloat16>(a);
    }
    return cudaErrorInvalidValue;
}

template <class T>
static cudaError_t launch_band_t(const LaunchArgs &a, float fsign) {
    const int threads = 64;
    const long long blocks = (a.P->nb + threads - 1) / threads;
    // programmatic dependent launch behind the last spreading of the chain
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3((unsigned)blocks);
    c.blockDim = dim3(threads);
    c.stream = a.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = attr;
    c.numAttrs = a.pdl ? 1 : 0;
    const DevState *ds = a.ds;
    float *band = a.band;
    if (a.thermal) return cudaLaunchKernelEx(&c, k_band_collide<T, true>, (T *)a.B, (T *)a.GB, *a.P, ds, band, fsign);
    return cudaLaunchKernelEx(&c, k_band_collide<T, false>, (T *)a.B, (T *)nullptr, *a.P, ds, band, fsign);
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
static cudaError_t launch_init_t(void *A, void *GA, void *A2, void *GA2, long long N, long long S, const float *fields,
                                 const float init[5], bool thermal, cudaStream_t s) {
    int threads = 256;
    long long blocks = (N + threads - 1) / threads;
    if (thermal)
        k_init<T, true><<<(unsigned)blocks, threads, 0, s>>>((T *)A, (T *)GA, (T *)A2, (T *)GA2, N, S, fields,
                                                             init[0], init[1], init[2], init[3], init[4]);
    else
        k_init<T, false><<<(unsigned)blocks, threads, 0, s>>>((T *)A, nullptr, (T *)A2, nullptr, N, S, fields,
                                                              init[0], init[1], init[2], init[3], init[4]);
    return cudaGetLastError();
}

cudaError_t launch_init(int storage, void *A, void *GA, void *A2, void *GA2, long long N, long long S,
                        const float *fields, const float init[5], bool thermal, cudaStream_t s) {
    switch (storage) {
    case 0: return launch_init_t<float>(A, GA, A2, GA2, N, S, fields, init, thermal, s);
    case 1: return launch_init_t<__half>(A, GA, A2, GA2, N, S, fields, init, thermal, s);
    case 2: return launch_init_t<__nv_bfloat16>(A, GA, A2, GA2, N, S, fields, init, thermal, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lbmk
