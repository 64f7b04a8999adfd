// lbm_stepv.cu -- the fused collide-stream step (the k_step update) with V
// consecutive x-cells per thread, V even: each population row segment is
// moved with one 4-, 8- or 16-byte load and one store instead of V scalar
// accesses, and the arithmetic runs on neighbouring cells in pairs with the
// packed FP32 instructions (Ar<float2>: one fma / mul / add updates both
// cells of a pair).
//
// Pull of link l for the cells x0 .. x0+V-1 of one row:
//   c_x(l) = 0: the source segment is aligned (same x, row y-c_y, z-c_z);
//   c_x(l) = +1: elements x0-1 .. x0+V-2 -- the aligned segment shifted by one
//     element, the missing one the last element of the lane to the left
//     (a warp shuffle; a word loaded beforehand where that lane holds another
//     row run);
//   c_x(l) = -1: elements x0+1 .. x0+V, the first element of the lane to the
//     right likewise.
// Cells on x = 0 / x = nx-1 then take their five x-crossing links from the
// x-face table (XFix).  Rows on a y or z face, and segments that overlap the
// IBM band where the band hand-off applies, take the one-cell-at-a-time
// path of k_step.  Both paths run the same explicitly rounded arithmetic
// (cell_state, collide_flow, collide_heat), so every kernel gives identical
// results.  Used for gather steps (not the first step, the moment export or
// the IBM near box) of solves without interior solids.
#include "lbm_internal.h"
#include "lbm_step.cuh"

namespace lbmk {

// Storage words: EPW elements of type T per 32-bit word, element e of the
// word at bits 16 e (little-endian element order).  Pair p of a segment is
// cells 2p, 2p+1: word p (16-bit types) or words 2p, 2p+1 (FP32).
template <class T>
struct Pk;
template <>
struct Pk<float> {
    static constexpr int EPW = 1;
    static __device__ __forceinline__ float2 get(const uint32_t *w, int p) {
        return make_float2(__uint_as_float(w[2 * p]), __uint_as_float(w[2 * p + 1]));
    }
    static __device__ __forceinline__ void put(uint32_t *w, int p, float2 v) {
        w[2 * p] = __float_as_uint(v.x);
        w[2 * p + 1] = __float_as_uint(v.y);
    }
    // (last element of a, first element of b)
    static __device__ __forceinline__ uint32_t join(uint32_t a, uint32_t) { return a; }
};
template <>
struct Pk<__half> {
    static constexpr int EPW = 2;
    static __device__ __forceinline__ float2 get(const uint32_t *w, int p) {
        __half2 h;
        memcpy(&h, &w[p], 4);
        return __half22float2(h);
    }
    static __device__ __forceinline__ void put(uint32_t *w, int p, float2 v) {
        const __half2 h = __floats2half2_rn(v.x, v.y);
        memcpy(&w[p], &h, 4);
    }
    static __device__ __forceinline__ uint32_t join(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
};
template <>
struct Pk<__nv_bfloat16> {
    static constexpr int EPW = 2;
    static __device__ __forceinline__ float2 get(const uint32_t *w, int p) {
        return make_float2(__uint_as_float(w[p] << 16), __uint_as_float(w[p] & 0xffff0000u));
    }
    static __device__ __forceinline__ void put(uint32_t *w, int p, float2 v) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
        memcpy(&w[p], &h, 4);
    }
    static __device__ __forceinline__ uint32_t join(uint32_t a, uint32_t b) { return __byte_perm(a, b, 0x5432); }
};

template <int NW>
__device__ __forceinline__ void ldv(const void *p, uint32_t (&w)[NW]) {
    if constexpr (NW == 1) {
        w[0] = __ldg(reinterpret_cast<const uint32_t *>(p));
    } else if constexpr (NW == 2) {
        const uint2 v = __ldg(reinterpret_cast<const uint2 *>(p));
        w[0] = v.x;
        w[1] = v.y;
    } else {
        static_assert(NW == 4, "1, 2 or 4 words");
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(p));
        w[0] = v.x;
        w[1] = v.y;
        w[2] = v.z;
        w[3] = v.w;
    }
}

template <int NW>
__device__ __forceinline__ void stv(void *p, const uint32_t (&w)[NW]) {
    if constexpr (NW == 1) {
        *reinterpret_cast<uint32_t *>(p) = w[0];
    } else if constexpr (NW == 2) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(w[0], w[1]);
    } else {
        *reinterpret_cast<uint4 *>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// The row segment of one link, pulled, from its aligned load w and the edge
// word e (loaded beforehand, branch-free): out[k] holds words of the pulled
// populations of the thread's cells.  For c_x = +1 the element left of the
// segment comes from the lane to the left (shuffle) or, where that lane
// holds another row run (needl), from e -- the word ending at that element;
// for c_x = -1 the element right of it likewise from the lane to the right
// or e, the word starting there.  Every lane of the warp calls this.
template <class T, int NW, int CX>
__device__ __forceinline__ void shift_row(const uint32_t (&w)[NW], uint32_t e, bool needl, bool needr,
                                          uint32_t (&out)[NW]) {
    constexpr int EPW = Pk<T>::EPW;
    if constexpr (CX == 0) {
#pragma unroll
        for (int k = 0; k < NW; k++) out[k] = w[k];
    } else if constexpr (CX > 0) {
        uint32_t prev = __shfl_up_sync(0xffffffffu, w[NW - 1], 1);
        prev = needl ? e : prev;
#pragma unroll
        for (int k = NW - 1; k > 0; k--) out[k] = Pk<T>::join(w[k - 1], w[k]);
        out[0] = Pk<T>::join(prev, w[0]);
    } else {
        uint32_t next = __shfl_down_sync(0xffffffffu, w[0], 1);
        next = needr ? e : next;
        if constexpr (EPW == 1) {
#pragma unroll
            for (int k = 0; k < NW - 1; k++) out[k] = w[k + 1];
            out[NW - 1] = next;
        } else {
#pragma unroll
            for (int k = 0; k < NW - 1; k++) out[k] = Pk<T>::join(w[k], w[k + 1]);
            out[NW - 1] = Pk<T>::join(w[NW - 1], next);
        }
    }
}

// Loads of the rows of NL links, all issued before any is used: the aligned
// segments (pc + row offset of the link), and for the x-shifted links the
// edge word from pl / pr -- the segment start moved to the word left / right
// of the segment where the lane needs it, else left in place (the load is
// then unused).
template <class T, int NW, int NL>
__device__ __forceinline__ void load_rows(const T *pc, const T *pl, const T *pr, const unsigned *rofs,
                                          uint32_t (&w)[NL][NW], uint32_t (&e)[NL]) {
#pragma unroll
    for (int l = 0; l < NL; l++) ldv<NW>(pc + rofs[l], w[l]);
#pragma unroll
    for (int l = 0; l < NL; l++) {
        if (cx(l) > 0) e[l] = __ldg(reinterpret_cast<const uint32_t *>(pl + rofs[l]));
        else if (cx(l) < 0) e[l] = __ldg(reinterpret_cast<const uint32_t *>(pr + rofs[l]));
        else e[l] = 0u;
    }
}

template <class T, int NW, int NL>
__device__ __forceinline__ void shift_rows(const uint32_t (&w)[NL][NW], const uint32_t (&e)[NL], bool needl,
                                           bool needr, uint32_t (&pk)[NL][NW]) {
#pragma unroll
    for (int l = 0; l < NL; l++) {
        if (cx(l) == 0) shift_row<T, NW, 0>(w[l], e[l], needl, needr, pk[l]);
        else if (cx(l) > 0) shift_row<T, NW, 1>(w[l], e[l], needl, needr, pk[l]);
        else shift_row<T, NW, -1>(w[l], e[l], needl, needr, pk[l]);
    }
}

// Resident blocks per SM asked of the compiler: the register budget that
// measured fastest for each segment width (an FP16 channel 256x128x128:
// two cells at 8 blocks 53.7 k MLUPS against 44.4 k unbounded).  BESIDE:
// the far region that runs beside the IBM kernels, where 7 blocks (more
// registers, fewer spills) measured faster on the sphere channel.
template <class T, int NP, bool THERMAL, bool BESIDE = false>
constexpr int stepv_min_blocks() {
    if constexpr (sizeof(T) == 4) return NP == 1 ? 6 : 1;
    if constexpr (THERMAL) return NP == 1 ? 4 : 1;
    if constexpr (BESIDE && NP == 1) return 7;
    return NP == 1 ? 8 : (NP == 2 ? 4 : 1);
}

template <class T, int NP, bool THERMAL, bool FORCED, bool BESIDE = false>
__global__ void __launch_bounds__(128, (stepv_min_blocks<T, NP, THERMAL, BESIDE>()))
    k_stepv(const T *__restrict__ A, T *__restrict__ B, const T *__restrict__ GA, T *__restrict__ GB,
            const __grid_constant__ StepParams P, DevState *__restrict__ ds, float *__restrict__ band, int region) {
    using A2 = Ar<float2>;
    constexpr int EPW = Pk<T>::EPW, V = 2 * NP, NW = V / EPW;
    // one thread per row segment of V cells: blockDim.x (a multiple of 32)
    // threads along a row, blockDim.y rows, so a warp never spans two rows
    const int lane = threadIdx.x & 31;
    const int per_row = P.nx / V;
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    const int x0 = seg * V;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    // nx is a multiple of V: a thread's cells are all inside or all outside
    const bool inrange = y < P.ny && seg < per_row;
    bool valid = inrange;
    // region 1 skips the near box (its x bounds are multiples of V)
    if (region == 1 && valid && x0 >= P.nlo[0] && x0 < P.nhi[0] && y >= P.nlo[1] && y < P.nhi[1] && z >= P.nlo[2] &&
        z < P.nhi[2])
        valid = false;
    // rows on a y or z face, periodic or not (the row offsets do not wrap),
    // and segments in the IBM band where its hand-off applies
    bool scalar = y == 0 || y == P.ny - 1 || z == 0 || z == P.nz - 1;
    if (region != 1 && P.band_on) {
        const int bx = ds->band_o[0], by = ds->band_o[1], bz = ds->band_o[2];
        scalar = scalar || (x0 + V > bx && x0 < bx + P.bsx && (unsigned)(y - by) < (unsigned)P.bsy &&
                            (unsigned)(z - bz) < (unsigned)P.bsz);
    }
    if (__any_sync(0xffffffffu, inrange && scalar)) {
        // the boundary-class path, cell by cell
#pragma unroll 1
        for (int i = 0; i < V; i++) {
            const int x = x0 + i;
            const long long cell = valid ? (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z) : 0;
            const int raw = valid ? ((x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) |
                                     (y == P.ny - 1 ? 8 : 0) | (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0))
                                  : 0;
            float f[Q], g[QT];
            gather_flow<T>(A, f, x, y, z, cell, raw, valid, true, 1, P);
            if (THERMAL) gather_heat<T>(GA, g, x, y, z, cell, raw, valid, true, 1, P);
            finish_cell<T, THERMAL, FORCED>(f, g, x, y, z, cell, valid, 1, 0, B, GB, P, ds, nullptr, band,
                                            region != 1);
        }
        return;
    }
    // lanes past the lattice read an interior row (x = 0, y = 1, z = 1)
    const unsigned c0 = inrange ? (unsigned)(x0 + P.nx * (y + P.ny * z)) : (unsigned)(P.nx * (1 + P.ny));
    // the lane to the left / right holds another row run (or none)
    const bool needl = lane == 0;
    const bool needr = lane == 31 || seg == per_row - 1;
    const int dl = needl ? -EPW : 0, dr = needr ? V : 0;
    uint32_t pk[Q][NW];
    uint32_t pg[THERMAL ? QT : 1][NW];
    {
        uint32_t w[Q][NW], e[Q];
        load_rows<T, NW, Q>(A + c0, A + c0 + dl, A + c0 + dr, P.rofs32, w, e);
        uint32_t wg[THERMAL ? QT : 1][NW], eg[THERMAL ? QT : 1];
        if constexpr (THERMAL) load_rows<T, NW, QT>(GA + c0, GA + c0 + dl, GA + c0 + dr, P.rofs32, wg, eg);
        shift_rows<T, NW, Q>(w, e, needl, needr, pk);
        if constexpr (THERMAL) shift_rows<T, NW, QT>(wg, eg, needl, needr, pg);
    }
    // x-face cells: their x-crossing links from the x-face table
    const bool xlo = valid && x0 == 0, xhi = valid && x0 + V == P.nx;
    float fl[5], fr[5], gl = 0.0f, gr = 0.0f;
    if (xlo) {
#pragma unroll
        for (int k = 0; k < 5; k++) fl[k] = xfix_link<T>(A, c0, P.xf[0], k);
        if (THERMAL) gl = xfix_heat<T>(GA, c0, P.xf[0]);
    }
    if (xhi) {
#pragma unroll
        for (int k = 0; k < 5; k++) fr[k] = xfix_link<T>(A, c0 + V - 1, P.xf[1], k);
        if (THERMAL) gr = xfix_heat<T>(GA, c0 + V - 1, P.xf[1]);
    }
    bool bad = false;
#pragma unroll
    for (int p = 0; p < NP; p++) {
        float2 f[Q], g[QT];
#pragma unroll
        for (int l = 0; l < Q; l++) f[l] = Pk<T>::get(pk[l], p);
        if (THERMAL) {
#pragma unroll
            for (int l = 0; l < QT; l++) g[l] = Pk<T>::get(pg[l], p);
        }
        if (p == 0 && xlo) {
#pragma unroll
            for (int j = 0; j < 5; j++) f[xpl(j)].x = fl[j];
            if (THERMAL) g[1].x = gl;
        }
        if (p == NP - 1 && xhi) {
#pragma unroll
            for (int j = 0; j < 5; j++) f[xml(j)].y = fr[j];
            if (THERMAL) g[2].y = gr;
        }
        float2 drho, ux, uy, uz, Fx, Fy, Fz, Tc;
        cell_state<float2, THERMAL, FORCED>(f, g, P, 0.5f, drho, ux, uy, uz, Fx, Fy, Fz, Tc);
        const float2 rho = A2::add(A2::splat(1.0f), drho);
        bad = bad || !(rho.x > 0.0f && rho.x < 100.0f) || !(rho.y > 0.0f && rho.y < 100.0f);
        collide_flow<float2, FORCED>(f, drho, ux, uy, uz, Fx, Fy, Fz, P.omega);
        if (THERMAL) collide_heat<float2, false>(g, Tc, ux, uy, uz, A2::splat(0.0f), P.omega_t);
#pragma unroll
        for (int l = 0; l < Q; l++) Pk<T>::put(pk[l], p, f[l]);
        if (THERMAL) {
#pragma unroll
            for (int l = 0; l < QT; l++) Pk<T>::put(pg[l], p, g[l]);
        }
    }
    const unsigned badw = __ballot_sync(0xffffffffu, valid && bad);
    if (badw && lane == 0) raise_status(&ds->status, ST_RHO_RANGE);
    if (!valid) return;
    T *pb = B + c0;
#pragma unroll
    for (int l = 0; l < Q; l++) stv<NW>(pb + P.sofs32[l], pk[l]);
    if (THERMAL) {
        T *pt = GB + c0;
#pragma unroll
        for (int l = 0; l < QT; l++) stv<NW>(pt + P.sofs32[l], pg[l]);
    }
}

// Blocks of 128 threads: blockDim.x the row's segments rounded up to whole
// warps (at most 128), blockDim.y rows; one z plane per blockIdx.z.
template <class T, int NP>
static cudaError_t launch_t(const LaunchArgs &a) {
    constexpr int V = 2 * NP;
    const StepParams &P = *a.P;
    const int per_row = P.nx / V;
    const int bx = per_row >= 128 ? 128 : ((per_row + 31) / 32) * 32;
    const dim3 blk(bx, 128 / bx, 1);
    const dim3 grd((per_row + bx - 1) / bx, (P.ny + blk.y - 1) / blk.y, P.nz);
    const T *A = (const T *)a.A, *GA = (const T *)a.GA;
    T *B = (T *)a.B, *GB = (T *)a.GB;
    if constexpr (sizeof(T) == 2 && NP == 1) {
        if (a.region == 1 && !a.thermal) {
            if (P.forced)
                k_stepv<T, NP, false, true, true><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, P, a.ds,
                                                                           a.band, a.region);
            else
                k_stepv<T, NP, false, false, true><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, P, a.ds,
                                                                            a.band, a.region);
            return cudaGetLastError();
        }
    }
    if (a.thermal)
        k_stepv<T, NP, true, true><<<grd, blk, 0, a.stream>>>(A, B, GA, GB, P, a.ds, a.band, a.region);
    else if (P.forced)
        k_stepv<T, NP, false, true><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, P, a.ds, a.band, a.region);
    else
        k_stepv<T, NP, false, false><<<grd, blk, 0, a.stream>>>(A, B, nullptr, nullptr, P, a.ds, a.band, a.region);
    return cudaGetLastError();
}

bool step_vec_usable(int storage, const StepParams &P, int vcells) {
    if (vcells < 2 || (vcells & 1) || !P.idx32 || P.solid != nullptr) return false;
    const int bytes = vcells * (storage == 0 ? 4 : 2);
    if (bytes != 4 && bytes != 8 && bytes != 16) return false;
    // aligned segments: whole rows of V cells, the stride a multiple of V
    return P.nx % vcells == 0 && P.S % vcells == 0 && P.ny >= 3 && P.nz >= 3;
}

cudaError_t launch_step_vec(int storage, const LaunchArgs &a) {
    switch (storage) {
    case 0: return a.vcells == 4 ? launch_t<float, 2>(a) : launch_t<float, 1>(a);
    case 1:
        return a.vcells == 8 ? launch_t<__half, 4>(a) : (a.vcells == 4 ? launch_t<__half, 2>(a) : launch_t<__half, 1>(a));
    case 2:
        return a.vcells == 8 ? launch_t<__nv_bfloat16, 4>(a)
                             : (a.vcells == 4 ? launch_t<__nv_bfloat16, 2>(a) : launch_t<__nv_bfloat16, 1>(a));
    }
    return cudaErrorInvalidValue;
}

}  // namespace lbmk
