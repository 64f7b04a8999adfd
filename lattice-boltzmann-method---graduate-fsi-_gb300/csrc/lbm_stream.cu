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
#include "lbm_collide.cuh"
#include "lbm_device.cuh"
#include "lbm_internal.h"

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
#pragma unroll
            for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(a + P.pofs32[l]) : 0.0f;
        } else {
#pragma unroll
            for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(a + P.pofs[l]) : 0.0f;
        }
        if (raw_cls & 3) {
            const ClassEntry &ce = P.cls[raw_cls & 3 & ~periodic_mask(P)];
#pragma unroll
            for (int l = 1; l < Q; l++) {
                if (cx(l) > 0 && (raw_cls & 1)) f[l] = pull_link<T>(A, l, x, y, z, cell, ce, P);
                if (cx(l) < 0 && (raw_cls & 2)) f[l] = pull_link<T>(A, l, x, y, z, cell, ce, P);
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
            const ClassEntry &ce = P.cls[raw_cls & 3 & ~periodic_mask(P)];
#pragma unroll
            for (int l = 1; l < QT; l++) {
                if (cx(l) > 0 && (raw_cls & 1)) g[l] = pull_heat_link<T>(G, l, x, y, z, cell, ce, P);
                if (cx(l) < 0 && (raw_cls & 2)) g[l] = pull_heat_link<T>(G, l, x, y, z, cell, ce, P);
            }
        }
        return;
    }
    const ClassEntry &ce = P.cls[raw_cls & ~periodic_mask(P)];
#pragma unroll
    for (int l = 0; l < QT; l++) g[l] = valid ? pull_heat_link<T>(G, l, x, y, z, cell, ce, P) : 0.0f;
}

// Everything after the gather of one cell: moments, optional moment output,
// band hand-off or collision, and the stores to B.
template <class T, bool THERMAL, bool FORCED>
__device__ __forceinline__ void finish_cell(float f[Q], float g[QT], int x, int y, int z, long long cell, bool valid,
                                            int gather, int export_only, T *__restrict__ B, T *__restrict__ GB,
                                            const StepParams &P, DevState *__restrict__ ds, float *__restrict__ mom,
                                            float *__restrict__ band, bool check_band = true) {
    const long long N = P.N;
    float drho, jx, jy, jz;
    moments_pairs(f, drho, jx, jy, jz);
    float Tc = 0.0f;
    float Fx = P.body[0], Fy = P.body[1], Fz = P.body[2];
    if (THERMAL) {
#pragma unroll
        for (int l = 0; l < QT; l++) Tc += g[l];
        Fx += P.gbeta[0] * (Tc - P.T0);
        Fy += P.gbeta[1] * (Tc - P.T0);
        Fz += P.gbeta[2] * (Tc - P.T0);
    }
    const float rho = 1.0f + drho;
    const float inv = inv_one_plus(drho);
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

    if (check_band && P.band_on) {
        const int bx = x - ds->band_o[0], by = y - ds->band_o[1], bz = z - ds->band_o[2];
        if ((unsigned)bx < (unsigned)P.bsx && (unsigned)by < (unsigned)P.bsy && (unsigned)bz < (unsigned)P.bsz) {
            const long long nb = P.nb;
            const long long b = bx + (long long)P.bsx * (by + (long long)P.bsy * bz);
#pragma unroll
            for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
            if (THERMAL) {
#pragma unroll
                for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
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
    collide_flow(f, drho, ux, uy, uz, Fx, Fy, Fz, FORCED, P.omega);
    if (P.idx32) {
        T *b = B + cell;
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(b + P.sofs32[l], f[l]);
    } else {
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
    }
    if (THERMAL) {
        collide_heat(g, Tc, ux, uy, uz, 0.0f, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
    }
}

// Fused step, direct global loads (any row length).  gather = 0 on the first
// step (A then holds the initial pre-collision populations in place);
// export_only = 1 computes and writes the moments of the gathered state
// without colliding or storing.
template <class T, bool THERMAL, bool FORCED>
__global__ void __launch_bounds__(256) k_step(const T *__restrict__ A, T *__restrict__ B, const T *__restrict__ GA,
                                              T *__restrict__ GB, const __grid_constant__ StepParams P,
                                              DevState *__restrict__ ds, float *__restrict__ mom,
                                              float *__restrict__ band, int gather, int export_only, int region) {
    // region 0: every cell; 1: all but the "near" box (the IBM band grown by
    // the one-cell pull stencil); 2: only the near box (the grid spans it)
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y * blockDim.y + threadIdx.y;
    int z = blockIdx.z;
    bool valid;
    if (region == 2) {
        x += ds->band_o[0] - 1;
        y += ds->band_o[1] - 1;
        z += ds->band_o[2] - 1;
        valid = x >= 0 && y >= 0 && z >= 0 && x < P.nx && y < P.ny && z < P.nz && x <= ds->band_o[0] + P.bsx &&
                y <= ds->band_o[1] + P.bsy && z <= ds->band_o[2] + P.bsz;
    } else {
        valid = (x < P.nx) && (y < P.ny);
        if (region == 1) {
            const int qx = x - (ds->band_o[0] - 1), qy = y - (ds->band_o[1] - 1), qz = z - (ds->band_o[2] - 1);
            if ((unsigned)qx < (unsigned)(P.bsx + 2) && (unsigned)qy < (unsigned)(P.bsy + 2) &&
                (unsigned)qz < (unsigned)(P.bsz + 2))
                valid = false;
        }
    }
    const long long cell = valid ? (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z) : 0;
    const int raw = valid ? ((x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                             (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0))
                          : 0;
    // With xface, x-face lanes of rows off the y/z faces stay on the plain
    // path and fix their x-crossing links themselves (gather_flow).
    const int rawrow = P.xface ? (raw & ~3) : raw;
    // the near box can start at a negative offset: keep those lanes idle
    const bool bwarp = __any_sync(0xffffffffu, rawrow != 0 || (region == 2 && !valid));
    float f[Q], g[QT];
    gather_flow<T>(A, f, x, y, z, cell, raw, valid, bwarp, gather, P);
    if (THERMAL) gather_heat<T>(GA, g, x, y, z, cell, raw, valid, bwarp, gather, P);
    finish_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, gather, export_only, B, GB, P, ds, mom, band,
                                    region != 1);
}

// ---------------------------------------------------------------------------
// Vector variant: each thread owns V = 8 / sizeof(T) consecutive cells of a
// row (4 for 16-bit storage, 2 for FP32) and pulls every population of the
// group with one aligned 8-byte load of the source row.  For links with
// c_x = +1 (-1) the group needs one more element on its left (right): it
// comes from the neighbouring lane's load through a warp shuffle, or for the
// first (last) lane of the warp from one extra scalar load.  So a thread
// keeps 19 x 8 bytes in flight.  Groups touching a domain face take the
// boundary-class path cell by cell.  Rows must be a multiple of V cells and
// x must not be periodic.
// ---------------------------------------------------------------------------
template <class T>
struct Vec8;
template <>
struct Vec8<float> {
    typedef float2 type;
    static constexpr int V = 2;
    static __device__ __forceinline__ type ld(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }
    static __device__ __forceinline__ float el(const type &v, int k) { return k == 0 ? v.x : v.y; }
    static __device__ __forceinline__ unsigned first_bits(const type &v) { return __float_as_uint(v.x); }
    static __device__ __forceinline__ unsigned last_bits(const type &v) { return __float_as_uint(v.y); }
    static __device__ __forceinline__ float from_bits(unsigned b) { return __uint_as_float(b); }
};
template <class H>
struct Vec8Half {
    typedef uint2 type;
    static constexpr int V = 4;
    static __device__ __forceinline__ type ld(const H *p) { return __ldg(reinterpret_cast<const uint2 *>(p)); }
    static __device__ __forceinline__ float cvt(unsigned short b) {
        H h;
        memcpy(&h, &b, 2);
        return St<H>::lds(&h);
    }
    static __device__ __forceinline__ float el(const type &v, int k) {
        const unsigned w = k < 2 ? v.x : v.y;
        return cvt((unsigned short)((k & 1) ? (w >> 16) : (w & 0xffffu)));
    }
    static __device__ __forceinline__ unsigned first_bits(const type &v) { return v.x & 0xffffu; }
    static __device__ __forceinline__ unsigned last_bits(const type &v) { return v.y >> 16; }
    static __device__ __forceinline__ float from_bits(unsigned b) { return cvt((unsigned short)b); }
};
template <>
struct Vec8<__half> : Vec8Half<__half> {};
template <>
struct Vec8<__nv_bfloat16> : Vec8Half<__nv_bfloat16> {};

template <class T, bool FORCED>
__global__ void __launch_bounds__(256) k_step_vec(const T *__restrict__ A, T *__restrict__ B,
                                                  const __grid_constant__ StepParams P, DevState *__restrict__ ds,
                                                  float *__restrict__ band, int region) {
    typedef Vec8<T> VT;
    constexpr int V = VT::V;
    const int lane = threadIdx.x & 31;
    const int x0 = V * (blockIdx.x * blockDim.x + threadIdx.x);
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool gvalid = x0 < P.nx && y < P.ny;
    const bool interior = gvalid && x0 >= 1 && x0 + V - 1 <= P.nx - 2 && y >= 1 && y <= P.ny - 2 && z >= 1 &&
                          z <= P.nz - 2;
    typename VT::type v[Q];
    float prev[Q], next[Q];
#pragma unroll
    for (int l = 0; l < Q; l++) {
        int sy = y - cy(l), sz = z - cz(l);
        if (P.periodic & 2) sy = sy < 0 ? sy + P.ny : (sy >= P.ny ? sy - P.ny : sy);
        if (P.periodic & 4) sz = sz < 0 ? sz + P.nz : (sz >= P.nz ? sz - P.nz : sz);
        const bool row_ok = gvalid && sy >= 0 && sy < P.ny && sz >= 0 && sz < P.nz;
        const T *rowp = A + l * P.S + (long long)P.nx * ((long long)sy + (long long)P.ny * sz);
        if (row_ok) {
            v[l] = VT::ld(rowp + x0);
        } else {
            memset(&v[l], 0, sizeof(v[l]));
        }
        if (cx(l) > 0) {
            const unsigned up = __shfl_up_sync(0xffffffffu, VT::last_bits(v[l]), 1);
            float pv = VT::from_bits(up);
            if (lane == 0) pv = (row_ok && x0 >= 1) ? St<T>::ld(rowp + x0 - 1) : 0.0f;
            prev[l] = pv;
        } else if (cx(l) < 0) {
            const unsigned dn = __shfl_down_sync(0xffffffffu, VT::first_bits(v[l]), 1);
            float nv = VT::from_bits(dn);
            if (lane == 31) nv = (row_ok && x0 + V < P.nx) ? St<T>::ld(rowp + x0 + V) : 0.0f;
            next[l] = nv;
        }
    }
    if (!gvalid) return;
#pragma unroll
    for (int k = 0; k < V; k++) {
        const int x = x0 + k;
        bool valid = true;
        if (region == 1) {
            const int qx = x - (ds->band_o[0] - 1), qy = y - (ds->band_o[1] - 1), qz = z - (ds->band_o[2] - 1);
            if ((unsigned)qx < (unsigned)(P.bsx + 2) && (unsigned)qy < (unsigned)(P.bsy + 2) &&
                (unsigned)qz < (unsigned)(P.bsz + 2))
                valid = false;
        }
        if (!valid) continue;
        const long long cell = (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z);
        float f[Q], g[QT];
        if (interior) {
#pragma unroll
            for (int l = 0; l < Q; l++) {
                if (cx(l) == 0)
                    f[l] = VT::el(v[l], k);
                else if (cx(l) > 0)
                    f[l] = k == 0 ? prev[l] : VT::el(v[l], k - 1);
                else
                    f[l] = k == V - 1 ? next[l] : VT::el(v[l], k + 1);
            }
        } else {
            const int raw = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                            (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0);
            gather_flow<T>(A, f, x, y, z, cell, raw, true, true, 1, P);
        }
        finish_cell<T, false, FORCED>(f, g, x, y, z, cell, true, 1, 0, B, nullptr, P, ds, nullptr, band);
    }
}

// ---------------------------------------------------------------------------
// Staged variant (warp-specialised, persistent).  A tile is TY whole rows
// (TY * nx cells) of one z plane.  Warp 0 is the producer: for every tile it
// arms the stage's "full" mbarrier with the byte count and issues, lane per
// population, one bulk asynchronous copy (cp.async.bulk, the TMA engine) of
// the source rows of that population -- the TY rows shifted by (cy, cz),
// widened by one 16-byte group on the side an x-link comes from -- into
// shared memory.  The other warps consume: each waits on "full", reads the
// pulled populations of its cells from shared memory, collides, stores to B
// and arrives on the stage's "empty" mbarrier, which the producer waits on
// before reusing the stage.  kStages tiles are in flight per CTA.  Cells on a
// domain face (and every cell of the first and last z plane, whose tiles
// stage nothing) take the boundary-class path from global memory.  All
// mbarrier waits are bounded; a wait that gives up sets ST_TIMEOUT.
// ---------------------------------------------------------------------------
constexpr int kStages = 4;
constexpr int kConsumers = 512;  // consumer threads per CTA (+ one producer warp)
constexpr long long kWaitLimit = 1ll << 24;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: true when the phase with this parity completed.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (long long i = 0; i < kWaitLimit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

template <class T, bool THERMAL>
__global__ void __launch_bounds__(kConsumers + 32, 1)
    k_step_tma(const T *__restrict__ A, T *__restrict__ B, const T *__restrict__ GA, T *__restrict__ GB,
               const __grid_constant__ StepParams P, DevState *__restrict__ ds, float *__restrict__ band, int TY,
               long long ntiles) {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int AL = 16 / (int)sizeof(T);
    constexpr int NQ = THERMAL ? Q + QT : Q;
    const int nx = P.nx;
    const int tcells = TY * nx;
    const int W = tcells + AL;
    const long long stage_elems = (long long)NQ * W;
    T *stage_base = reinterpret_cast<T *>(smem);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + ((kStages * stage_elems * (long long)sizeof(T) + 15) / 16) * 16);
    uint64_t *empty = full + kStages;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int ncw = kConsumers / 32;  // consumer warps
    if (tid == 0) {
        for (int st = 0; st < kStages; st++) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], ncw);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long long G = gridDim.x;
    const long long t0 = blockIdx.x;
    const long long nloc = t0 < ntiles ? (ntiles - t0 + G - 1) / G : 0;
    const int tiles_y = P.ny / TY;

    if (warp == 0) {
        // ---------------- producer ----------------
        for (long long k = 0; k < nloc; k++) {
            const int st = (int)(k % kStages);
            if (k >= kStages) {
                bool ok = true;
                if (lane == 0) ok = mbar_wait_bounded(&empty[st], (uint32_t)(((k / kStages) - 1) & 1));
                ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
                if (!ok) {
                    if (lane == 0) atomicOr(&ds->status, ST_TIMEOUT);
                    return;
                }
            }
            const long long t = t0 + k * G;
            const int y0 = (int)(t % tiles_y) * TY;
            const int z = (int)(t / tiles_y);
            const bool edge_plane = (z == 0 || z == P.nz - 1);
            const uint32_t full_b = (uint32_t)((tcells + AL) * sizeof(T)), narrow_b = (uint32_t)(tcells * sizeof(T));
            if (lane == 0) {
                uint32_t bytes = 0;
                if (!edge_plane) {
#pragma unroll
                    for (int q = 0; q < NQ; q++) {
                        const int l = q < Q ? q : q - Q;
                        bytes += cx(l) != 0 ? full_b : narrow_b;
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive_expect_tx(&full[st], bytes);
            }
            __syncwarp();
            if (!edge_plane && lane < NQ) {
                const int q = lane;
                const int l = q < Q ? q : q - Q;
                const T *base = q < Q ? A : GA;
                const int clx = cx(l), cly = cy(l), clz = cz(l);
                const long long start = (clx > 0 ? -AL : 0) +
                                        (long long)nx * ((long long)(y0 - cly) + (long long)P.ny * (z - clz));
                bulk_g2s(stage_base + st * stage_elems + (long long)q * W, base + l * P.S + start,
                         clx != 0 ? full_b : narrow_b, &full[st]);
            }
        }
        return;
    }
    // ---------------- consumers ----------------
    const int ct = tid - 32;
    for (long long k = 0; k < nloc; k++) {
        const int st = (int)(k % kStages);
        const uint32_t parity = (uint32_t)((k / kStages) & 1);
        bool ok = true;
        if (lane == 0) ok = mbar_wait_bounded(&full[st], parity);
        ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
        if (!ok) {
            if (lane == 0) atomicOr(&ds->status, ST_TIMEOUT);
            return;
        }
        mbar_try_wait(&full[st], parity);  // per-thread acquire of the staged data
        const long long t = t0 + k * G;
        const int y0 = (int)(t % tiles_y) * TY;
        const int z = (int)(t / tiles_y);
        const T *sb = stage_base + st * stage_elems;
        for (int c = ct; c < tcells; c += kConsumers) {
            const int y = y0 + c / nx, x = c - (c / nx) * nx;
            const long long cell = (long long)x + (long long)nx * ((long long)y + (long long)P.ny * z);
            const int raw = (x == 0 ? 1 : 0) | (x == nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                            (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0);
            float f[Q], g[QT];
            if (raw == 0) {
#pragma unroll
                for (int l = 0; l < Q; l++) {
                    const int off = cx(l) > 0 ? AL - 1 : (cx(l) < 0 ? 1 : 0);
                    f[l] = St<T>::lds(sb + l * W + c + off);
                }
                if (THERMAL) {
#pragma unroll
                    for (int l = 0; l < QT; l++) {
                        const int off = cx(l) > 0 ? AL - 1 : (cx(l) < 0 ? 1 : 0);
                        g[l] = St<T>::lds(sb + (Q + l) * W + c + off);
                    }
                }
            } else {
                gather_flow<T>(A, f, x, y, z, cell, raw, true, true, 1, P);
                if (THERMAL) gather_heat<T>(GA, g, x, y, z, cell, raw, true, true, 1, P);
            }
            finish_cell<T, THERMAL, true>(f, g, x, y, z, cell, true, 1, 0, B, GB, P, ds, nullptr, band);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
    }
}

// Collision of the IBM band cells, after the forcing iterations: rho and the
// unforced velocity from k_step, the accumulated IBM force Ft (band[7..9])
// and heat source (band[11]).  u = u_unf + Ft / (2 rho) and F = Fb + sign Ft
// (sign = -1 reproduces lbm.cpp:1347-1352); T = T_unf + Qt / 2.
// 64-thread blocks of at most 64 registers: they fit beside the far-region
// collide-stream blocks (which leave 4096 registers per SM) when overlapped.
template <class T, bool THERMAL>
__global__ void __launch_bounds__(64, 16) k_band_collide(T *__restrict__ B, T *__restrict__ GB,
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
    const long long nb = P.nb;
    const long long cell = x + (long long)P.nx * (y + (long long)P.ny * z);
    float f[Q];
#pragma unroll
    for (int l = 0; l < Q; l++) f[l] = St<T>::ld(B + l * P.S + cell);
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
    for (int l = 0; l < Q; l++) St<T>::st(B + l * P.S + cell, f[l]);
    if (THERMAL) {
        float g[QT];
#pragma unroll
        for (int l = 0; l < QT; l++) g[l] = St<T>::ld(GB + l * P.S + cell);
        const float Qt = band[11 * nb + b];
        const float Tc = band[10 * nb + b] + 0.5f * Qt;
        collide_heat(g, Tc, ux, uy, uz, Qt, P.omega_t);
#pragma unroll
        for (int l = 0; l < QT; l++) St<T>::st(GB + l * P.S + cell, g[l]);
    }
}

// Initial populations (LBM::Init, lbm.cpp:31-57): f = feq3(rho, u) stored
// shifted, g = geq(T, u); from uniform values or per-cell host fields.
template <class T, bool THERMAL>
__global__ void k_init(T *__restrict__ A, T *__restrict__ GA, long long N, long long S,
                       const float *__restrict__ fields, float rho0, float ux0, float uy0, float uz0, float T0) {
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
        St<T>::st(A + l * S + c, wf(l) * (drho + rho * p3));
    }
    if (THERMAL) {
#pragma unroll
        for (int l = 0; l < QT; l++) {
            const float cu = cx(l) * ux + cy(l) * uy + cz(l) * uz;
            St<T>::st(GA + l * S + c, wtf(l) * Tc * (1.0f + 4.0f * cu));
        }
    }
}

// ---------------------------------------------------------------------------
// Host-side launchers.
// ---------------------------------------------------------------------------
template <class T>
static cudaError_t launch_step_t(const LaunchArgs &a) {
    const TmaPlan &tp = a.tma;
    if (tp.enabled && a.gather && !a.export_only && a.mom == nullptr && a.region == 0) {
        if (a.thermal)
            k_step_tma<T, true><<<tp.grid, kConsumers + 32, tp.smem, a.stream>>>(
                (const T *)a.A, (T *)a.B, (const T *)a.GA, (T *)a.GB, *a.P, a.ds, a.band, tp.ty, tp.ntiles);
        else
            k_step_tma<T, false><<<tp.grid, kConsumers + 32, tp.smem, a.stream>>>(
                (const T *)a.A, (T *)a.B, nullptr, nullptr, *a.P, a.ds, a.band, tp.ty, tp.ntiles);
        return cudaGetLastError();
    }
    if (a.vec && a.gather && !a.export_only && a.mom == nullptr && !a.thermal && a.region != 2) {
        constexpr int V = Vec8<T>::V;
        const int groups = a.P->nx / V;
        const int tx = groups >= 128 ? 128 : (groups >= 64 ? 64 : 32);
        dim3 blk(tx, 256 / tx, 1);
        dim3 grd((groups + tx - 1) / tx, (a.P->ny + blk.y - 1) / blk.y, a.P->nz);
        if (a.P->forced)
            k_step_vec<T, true><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, *a.P, a.ds, a.band, a.region);
        else
            k_step_vec<T, false><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, *a.P, a.ds, a.band, a.region);
        return cudaGetLastError();
    }
    dim3 blk(a.tx, a.ty, 1);
    dim3 grd((a.P->nx + a.tx - 1) / a.tx, (a.P->ny + a.ty - 1) / a.ty, a.P->nz);
    if (a.region == 2) grd = dim3((a.P->bsx + 2 + a.tx - 1) / a.tx, (a.P->bsy + 2 + a.ty - 1) / a.ty, a.P->bsz + 2);
    const bool forced = a.P->forced != 0;
    if (a.thermal)
        k_step<T, true, true><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, (const T *)a.GA, (T *)a.GB, *a.P,
                                                         a.ds, a.mom, a.band, a.gather, a.export_only, a.region);
    else if (forced)
        k_step<T, false, true><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, nullptr, nullptr, *a.P, a.ds,
                                                          a.mom, a.band, a.gather, a.export_only, a.region);
    else
        k_step<T, false, false><<<grd, blk, 0, a.stream>>>((const T *)a.A, (T *)a.B, nullptr, nullptr, *a.P, a.ds,
                                                           a.mom, a.band, a.gather, a.export_only, a.region);
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

template <class T, bool THERMAL>
static cudaError_t plan_t(const StepParams &P, int ty_pref, TmaPlan &tp) {
    constexpr int AL = 16 / (int)sizeof(T);
    constexpr int NQ = THERMAL ? Q + QT : Q;
    tp.enabled = 0;
    if (P.nx % AL != 0 || P.nx < 2 || P.ny < 3 || P.nz < 3) return cudaSuccess;
    // rows per tile: about 40 KB of staged populations, dividing ny
    int ty = ty_pref > 0 ? ty_pref : (int)(40960 / ((size_t)NQ * P.nx * sizeof(T)));
    if (ty < 1) ty = 1;
    if (ty > P.ny) ty = P.ny;
    while (P.ny % ty != 0) ty--;
    const size_t stage_bytes = (size_t)NQ * ((size_t)ty * P.nx + AL) * sizeof(T);
    const size_t smem = ((kStages * stage_bytes + 15) / 16) * 16 + 2 * kStages * sizeof(uint64_t);
    if (smem > 220 * 1024) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(k_step_tma<T, THERMAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, dev = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step_tma<T, THERMAL>, kConsumers + 32, smem)) !=
        cudaSuccess)
        return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if (per_sm < 1) return cudaSuccess;
    tp.ty = ty;
    tp.ntiles = (long long)(P.ny / ty) * P.nz;
    tp.smem = smem;
    long long g = (long long)per_sm * sms;
    tp.grid = (int)(g < tp.ntiles ? g : tp.ntiles);
    tp.per_sm = per_sm;
    tp.enabled = 1;
    return cudaSuccess;
}

cudaError_t plan_tma(int storage, bool thermal, const StepParams &P, int ty_pref, TmaPlan &tp) {
    switch (storage) {
    case 0: return thermal ? plan_t<float, true>(P, ty_pref, tp) : plan_t<float, false>(P, ty_pref, tp);
    case 1: return thermal ? plan_t<__half, true>(P, ty_pref, tp) : plan_t<__half, false>(P, ty_pref, tp);
    case 2:
        return thermal ? plan_t<__nv_bfloat16, true>(P, ty_pref, tp) : plan_t<__nv_bfloat16, false>(P, ty_pref, tp);
    }
    return cudaErrorInvalidValue;
}

template <class T>
static cudaError_t launch_band_t(const LaunchArgs &a, float fsign) {
    const int threads = 64;
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
static cudaError_t launch_init_t(void *A, void *GA, long long N, long long S, const float *fields, const float init[5],
                                 bool thermal, cudaStream_t s) {
    int threads = 256;
    long long blocks = (N + threads - 1) / threads;
    if (thermal)
        k_init<T, true><<<(unsigned)blocks, threads, 0, s>>>((T *)A, (T *)GA, N, S, fields, init[0], init[1],
                                                             init[2], init[3], init[4]);
    else
        k_init<T, false><<<(unsigned)blocks, threads, 0, s>>>((T *)A, nullptr, N, S, fields, init[0], init[1],
                                                              init[2], init[3], init[4]);
    return cudaGetLastError();
}

cudaError_t launch_init(int storage, void *A, void *GA, long long N, long long S, const float *fields,
                        const float init[5], bool thermal, cudaStream_t s) {
    switch (storage) {
    case 0: return launch_init_t<float>(A, GA, N, S, fields, init, thermal, s);
    case 1: return launch_init_t<__half>(A, GA, N, S, fields, init, thermal, s);
    case 2: return launch_init_t<__nv_bfloat16>(A, GA, N, S, fields, init, thermal, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace lbmk
