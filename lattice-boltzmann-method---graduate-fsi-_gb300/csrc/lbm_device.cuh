// lbm_device.cuh -- device-side definitions shared by the LBM kernels.
//
// Lattice: D3Q19 in the reference order (LBM.h:542-552) so that population l
// on the device is population l of the reference's LATTICE::f[]; D3Q7 thermal
// links are D3Q19 links 0..6.
//
// Storage: populations are kept shifted, f~ = f - w (and g unshifted), in
// float, __half or __nv_bfloat16, structure-of-arrays: pop[l * S + cell] with
// cell = x + nx * (y + ny * z) over interior cells only and a padded stride
// S >= N.  All arithmetic is FP32.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace lbmk {

constexpr int Q = 19;
constexpr int QT = 7;

__host__ __device__ constexpr int cx(int l) {
    constexpr int v[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
    return v[l];
}
__host__ __device__ constexpr int cy(int l) {
    constexpr int v[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
    return v[l];
}
__host__ __device__ constexpr int cz(int l) {
    constexpr int v[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
    return v[l];
}
__host__ __device__ constexpr int opp(int l) {
    constexpr int v[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
    return v[l];
}
// The links with c_x = +1 (xpl) and c_x = -1 (xml), in link order: the five
// links a cell on x = 0, respectively x = nx-1, pulls across its x face.
__host__ __device__ constexpr int xpl(int k) {
    constexpr int v[5] = {1, 7, 9, 13, 15};
    return v[k];
}
__host__ __device__ constexpr int xml(int k) {
    constexpr int v[5] = {2, 8, 10, 14, 16};
    return v[k];
}
__host__ __device__ constexpr float wf(int l) {
    return l == 0 ? (1.0f / 3.0f) : (l < 7 ? (1.0f / 18.0f) : (1.0f / 36.0f));
}
__host__ __device__ constexpr double wd(int l) { return l == 0 ? (1.0 / 3.0) : (l < 7 ? (1.0 / 18.0) : (1.0 / 36.0)); }
__host__ __device__ constexpr float wtf(int l) { return l == 0 ? 0.25f : 0.125f; }

// Storage conversions.
template <class T>
struct St;
template <>
struct St<float> {
    static __device__ __forceinline__ float ld(const float *p) { return __ldg(p); }
    static __device__ __forceinline__ float lds(const float *p) { return *p; }
    static __device__ __forceinline__ void st(float *p, float v) { *p = v; }
};
template <>
struct St<__half> {
    static __device__ __forceinline__ float ld(const __half *p) { return __half2float(__ldg(p)); }
    static __device__ __forceinline__ float lds(const __half *p) { return __half2float(*p); }
    static __device__ __forceinline__ void st(__half *p, float v) { *p = __float2half_rn(v); }
};
template <>
struct St<__nv_bfloat16> {
    static __device__ __forceinline__ float ld(const __nv_bfloat16 *p) { return __bfloat162float(__ldg(p)); }
    static __device__ __forceinline__ float lds(const __nv_bfloat16 *p) { return __bfloat162float(*p); }
    static __device__ __forceinline__ void st(__nv_bfloat16 *p, float v) { *p = __float2bfloat16_rn(v); }
};

// Bit of a packed per-cell mask (32 cells per word, cell index order).
__device__ __forceinline__ bool mask_bit(const uint32_t *__restrict__ m, long long cell) {
    return (__ldg(m + (cell >> 5)) >> (cell & 31)) & 1u;
}

// Boundary class of a cell: which ghost faces it touches.  Bit 2a is the low
// face of axis a, bit 2a+1 the high face; periodic axes never set bits.
struct ClassEntry {
    uint32_t bb;      // link l pulls from a wall: bounce-back
    uint32_t eq;      // link l pulls from an inlet/outlet-equilibrium ghost
    uint32_t zg;      // link l pulls from a zero-gradient outlet ghost
    uint32_t tdir;    // thermal: wall link with Dirichlet temperature
    float val[Q];     // bb: +2 w (c.u_w)/cs^2;  eq: feq(face) - w
    float tval[QT];   // thermal: eq: geq(face);  tdir: 2 w T_wall
};

// The five x-crossing links of a cell on x = 0 (face 0: links with c_x = +1)
// or x = nx-1 (face 1: c_x = -1) in a row off the y/z faces, as the
// boundary-class rule resolves them for that face: value = add (an
// equilibrium ghost, bit k of eq) or sgn * A[cell + ofs] + add, rounded
// once (bounce-back: the cell's own opposite population plus the wall term;
// a periodic or zero-gradient pull: the wrapped or clamped source, add 0).
// The D3Q7 link of the face likewise (t*).
struct XFix {
    unsigned ofs[5];
    float sgn[5];
    float add[5];
    unsigned eq;
    unsigned tofs;
    float tsgn, tadd;
    int teq;
};

// Per-launch parameters, passed by value as a __grid_constant__.
struct StepParams {
    int nx, ny, nz;
    int periodic;          // bit a: axis a periodic
    long long N;           // nx * ny * nz
    long long S;           // population stride (>= N + one tile of slack, see lbm_abi.cu)
    long long pofs[Q];     // l * S - (cx + nx (cy + ny cz)): pull offset of link l from the cell
    unsigned pofs32[Q];    // the same as 32-bit words when idx32 (never negative)
    unsigned sofs32[Q];    // l * S as 32-bit words when idx32
    unsigned rofs32[Q];    // l * S - nx (cy + ny cz): the source row of link l, same x (when idx32)
    int idx32;             // 19 S < 2^31 and a safe cell exists: 32-bit element indices
    unsigned safe_cell;    // a cell whose whole pull stencil is inside the lattice: idle
                           // lanes load from it instead of being predicated off
    int xface;            // x-face lanes stay on the plain path and fix their x-crossing links
    float omega;           // dt / tau
    float omega_t;         // dt / tau_g
    float body[3];         // uniform body force
    float gbeta[3];        // Boussinesq: F += gbeta (T - T0)
    float T0;
    int forced;            // body force or buoyancy present
    // IBM band (box of interior cells whose collision waits for the IBM)
    int band_on;
    int bsx, bsy, bsz;     // band extent
    long long nb;          // bsx * bsy * bsz
    int nlo[3], nhi[3];    // near box of a fixed body: band grown by one cell, rounded out to tiles
    long long *bandq;      // [4][nb] accumulated IBM force (x, y, z) and heat, fixed point (to_fx)
    // interior solid cells (staircase bodies), or null
    const uint32_t *solid;  // bit per interior cell: stationary solid (bounce-back on its links)
    const uint32_t *nearw;  // bit per interior cell: a solid, or a neighbour of one
    float *mea;             // per-block momentum-exchange partial sums [blocks][3], or null
    XFix xf[2];             // x-face links of interior rows (when idx32)
    ClassEntry cls[64];
};

// Device-resident state of one solve: status word, step counter, band
// origin and the FP64 rigid body.
struct DevState {
    uint32_t status;
    long long mea_step;     // reference step of the next momentum-exchange record
    int band_o[3];          // band origin (interior cell coordinates)
    long long step;         // steps completed on the device
    long long hist_cap;
    double body_xc[3], body_v[3], body_om[3];
    double body_dxc[3];
    double internal_prev[6];  // fluid momentum / angular momentum inside the body, previous step
    int have_prev;
    double body_v_prev[3], body_om_prev[3];  // previous step's velocities (virtual-mass term)
};

enum : uint32_t {
    ST_RHO_RANGE = 1u,      // rho outside (0, 100) or NaN (lbm.cpp:772-775)
    ST_BAND_EDGE = 2u,      // a marker stencil left the band / interior
    ST_NONFINITE_FORCE = 4u,
    ST_FEQ_NEG = 8u,
    ST_TIMEOUT = 16u,       // a bounded mbarrier wait gave up
    ST_T_RANGE = 32u,       // ENERGY: T outside (0, 100) or NaN (lbm.cpp:794-797)
};

__device__ __forceinline__ int cell_class(int x, int y, int z, const StepParams &P) {
    int c = (x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
            (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0);
    int pm = ((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0) | ((P.periodic & 4) ? 48 : 0);
    return c & ~pm;
}

// The spreading accumulates in 64-bit fixed point: v * 2^44 (an exact
// scaling) rounded to an integer, so the sum of a node's contributions is
// the same in whatever order the atomics land; read back with one rounding
// to FP32.  |v| stays far below 2^19 for any finite forcing.
// Set a status bit from one lane: a plain read first, so that a diverged
// solve, where every warp of every step finds a bad cell, sends one atomic
// per warp only until the bit is set instead of on every step.
__device__ __forceinline__ void raise_status(uint32_t *status, uint32_t bit) {
    if ((*reinterpret_cast<volatile uint32_t *>(status) & bit) == 0u) atomicOr(status, bit);
}

constexpr float kFxScale = 17592186044416.0f;  // 2^44
__device__ __forceinline__ long long to_fx(float v) { return __float2ll_rn(v * kFxScale); }
__device__ __forceinline__ float from_fx(long long q) { return __ll2float_rn(q) * (1.0f / kFxScale); }

// 4-point Peskin delta, kernel(r) of lbm.cpp:1095-1102, in FP32.
__device__ __forceinline__ float peskin(float r) {
    float a = fabsf(r);
    if (a <= 1.0f) return (3.0f - 2.0f * a + sqrtf(fmaxf(1.0f + 4.0f * a - 4.0f * r * r, 0.0f))) * 0.125f;
    if (a <= 2.0f) return (5.0f - 2.0f * a - sqrtf(fmaxf(-7.0f + 12.0f * a - 4.0f * r * r, 0.0f))) * 0.125f;
    return 0.0f;
}

}  // namespace lbmk
