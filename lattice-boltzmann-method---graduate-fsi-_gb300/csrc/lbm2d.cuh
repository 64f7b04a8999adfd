// lbm2d.cuh -- device-side definitions of the D2Q9 solver (lbm2d.cu).
//
// Lattice: D2Q9 in the reference order (LBM.h, the D2Q9 tables:
// c = (0,0) (1,0) (0,1) (-1,0) (0,-1) (1,1) (-1,1) (-1,-1) (1,-1)), so that
// population l on the device is population l of the reference's
// LATTICE::f[] in a D2Q9 build.  Populations are kept shifted (f - w), SoA
// pop[l * S + cell], cell = x + nx * y over the interior of the reference's
// single computational layer k = 1.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace l2d {

constexpr int Q9 = 9;

__host__ __device__ constexpr int cx9(int l) {
    constexpr int v[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
    return v[l];
}
__host__ __device__ constexpr int cy9(int l) {
    constexpr int v[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
    return v[l];
}
__host__ __device__ constexpr int opp9(int l) {
    constexpr int v[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
    return v[l];
}
__host__ __device__ constexpr float w9f(int l) { return l == 0 ? (4.0f / 9.0f) : (l < 5 ? (1.0f / 9.0f) : (1.0f / 36.0f)); }
__host__ __device__ constexpr double w9d(int l) { return l == 0 ? (4.0 / 9.0) : (l < 5 ? (1.0 / 9.0) : (1.0 / 36.0)); }

// Boundary class of a face cell (bit 0: x = 0, 1: x = nx-1, 2: y = 0,
// 3: y = ny-1; periodic axes set none): per link, bounce-back from a wall,
// the face equilibrium, or a zero-gradient pull.
struct Class2 {
    uint32_t bb, eq, zg;
    float val[Q9];  // bb: +6 w (c . u_wall);  eq: feq(face) - w
};

struct Params2 {
    int nx, ny;
    long long N, S;
    float omega;
    float body[2];
    int forced;
    int periodic;   // bit 0: x, bit 1: y
    int pofs[Q9];   // plain pull offset of link l: -(cx + nx cy)
    Class2 cls[16];
    // the classes once the walls move at F/2 (lbm_config.wall_force: the
    // reference's Poiseuille_Flow sets the body force on every cell, walls
    // included, lbm.cpp:800-801); used from the third streaming on
    Class2 cls_w[16];
    int bsx, bsy;   // allocated box (band) extent; band arrays are [5][bsx * bsy]
    long long nb;
    int band_on;
    // interior solid cells (staircase bodies): per cell, bit l set when the
    // source x - c_l of link l is a solid, bit 15 when the cell is one
    const uint16_t *links;
};

constexpr uint32_t kSolidCell = 0x8000u;
constexpr uint32_t kSolidLinks = 0x1FFu;

// The reference's ENERGY model (LBM.h:58) on a D2Q9 handle: temperature
// populations g on the flow lattice, stored shifted (g - w T_ref) in the
// storage type of f.  Per boundary class: the links whose source is a
// Dirichlet wall, P(c_opp . u_w) - 1 of their wall equilibrium, and the wall
// temperature (Determine_Wall_Temperature, lbm.cpp:965-981) at the first
// streaming (the set-up wall T) and at later ones (the wall's own sum g
// after the first MacroProp).
struct Energy2 {
    float inv_tau_g;     // 1 / tau_g
    float tg_fac;        // (tau_g - 1/2) / (cs2 tau_g)
    float inv_cp;        // 1 / cp
    float two_nu;        // 2 nu, nu = cs2 (tau - 1/2)
    float s_fac;         // -1 / (2 tau cs2): S = s_fac / rho * sum c c (f - feq)
    float T_ref;         // shift of the stored g; the uniform set-up T
    uint32_t dir[16];    // links l of a class whose source is a Dirichlet wall
    float pm1[16][Q9];   // P(c_opp(l) . u_w) - 1 of the wall equilibrium
    float pm1_w[16][Q9]; // the same with the walls moving at F/2 (cls_w)
    float tw[16][2];     // wall T (first streaming, later)
    float dtw[16][2];    // wall T - T_ref
    // Neumann walls (type_Energy TYPE_Q, j.n = 0; Determine_Twall_Neumann,
    // lbm.cpp:983-1028) and adiabatic walls (any other type_Energy: their
    // links are never written and keep the Init value), per class
    uint32_t neu[16];    // links whose source is a Neumann wall
    uint32_t adi[16];    // links whose source is an adiabatic wall
    float cn[16][Q9];    // c_l . n, n the mean direction of the class's wall links
    float nk[16];        // sum over the other links of w_l c_l . n (the T_ref shift)
    float nd[16];        // sum over the wall links of w_l P3(u_w . c_l) c_l . n
    float nq[16][Q9];    // P2(-u_w . c_l) of a wall link l: its g over w_l rho T_w
    float *gold;         // [Q9][S] of the wall cells: last sweep's values, the Init values
};

// Device state of a D2Q9 solve.  The body kinematics are those of IBLBM
// (lbm.cpp:1136-1167): V_CM of the current step and of the step before, the
// centre, and the box [floor(c - D), ceil(c + D)] of the current step.
struct State2 {
    uint32_t status;
    int box_lo[2];      // device cell of the box's lower corner (reference node - 1)
    int box_w, box_h;   // box extent of the current step
    long long ibm_step; // reference step of the current IBM pass (1-based)
    double center[3];
    double V[3], Vold[3];
    int lists_ok;       // spreading lists valid (fixed body)
    int fbox[4];        // box of the latest IBM pass {x0, y0, w, h}: the extent of Ibm2::boxF
    long long hist_cap;
};

}  // namespace l2d
