// LBM.h -- drop-in host facade with the reference's class surface
// (DestinyFlow01/Lattice-Boltzmann-Method---Graduate-FSI-, LBM.h:528-761),
// running the time step on the GPU through the C ABI (include/lbmgpu.h).
//
// What stays the same for a caller of the reference:
//   - the cell types TYPE_F .. TYPE_Q (LBM.h:505-515), the D3Q19 tables
//     cx/cy/cz/w/opposite in the reference order (LBM.h:542-552), or the D2Q9
//     ones when built with -DD2Q9 (LBM.h:529-539);
//   - class LATTICE with type/density/ux/uy/uz/f/f_star/F/Fm (LBM.h:558-597)
//     and the public LATTICE ***fluid array of (Nx+2)(Ny+2)(Nz+2) cells;
//   - class MARKER (LBM.h:600-616) and the free functions kernel,
//     NearestLatticeCoordinate, Calc_AverageDensity and IBLBM (LBM.h:674-688);
//   - class LBM: LBM(Nx, Ny, Nz, tau), Init, Collision, Streaming, MacroProp,
//     ConvLBM, Calc_feq, Determine_Wall_Velocity, getNx/getNy/getNz/getTAU.
// What changes:
//   - Init() reads fluid[..].type / density / ux.. (the set-up the reference's
//     main_setup_* functions write), builds the device configuration and
//     uploads the state; from then on the populations live on the GPU;
//   - Collision() + Streaming() run one fused step on the device (Collision
//     only records that a collision is pending); MacroProp() is fused into
//     the step and here only marks the host mirror stale;
//   - sync_to_host() fills fluid[..].density/ux/uy/uz (and T; with ENERGY
//     also q) with the MacroProp moments before output code reads them;
//   - IBLBM registers the markers with the device on its first call; the
//     forcing runs inside the next step and Cl/Cd are appended after it.
// Compile-time choices of the reference (#define D3Q19, IBM scheme, m_max,
// D, u_max ...) become fields of lbm_options.
#pragma once
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "../../../include/lbmgpu.h"

#ifndef TYPE_F
#define TYPE_F 0    // fluid domain
#define TYPE_S 1    // (stationary or moving) solid boundary
#define TYPE_OUT 2  // outflow boundary
#define TYPE_IN 3   // inflow boundary
#define TYPE_P 4    // periodic boundary
#define TYPE_L 5    // slip boundary
#define TYPE_T 6    // Dirichlet temperature
#define TYPE_Q 7    // Neumann heat flux
#endif

// truncated PI of the reference (LBM.h:74)
static const double PI = 3.14159265;

#if defined D2Q9
// D2Q9 in the reference order (LBM.h:529-539); the computational layer is
// k = 1 of fluid[Nx+2][Ny+2][3]
const int ndim = 2;
const int npop = 9;
const int cx[npop] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int cy[npop] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int cz[npop] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
const double w[npop] = {4.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
const int opposite[npop] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
#else
const int ndim = 3;
const int npop = 19;
const int cx[npop] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
const int cy[npop] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
const int cz[npop] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
const double w[npop] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                        1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                        1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
const int opposite[npop] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
#endif

// Run-time replacement of the reference's compile-time configuration.
struct lbm_options {
    int storage = LBM_STORE_F32;  // LBM_STORE_F32 / F16 / BF16
    int m_max = 5;                // implicit IBM iterations (LBM.h:357)
    int literal_sign = 0;         // 1: the reference's force-sign convention (lbm.cpp:1347-1352)
    double rho0 = 1.0;            // LBM.h:80
    double u_max = 0.05;          // reference velocity for Cl/Cd
    double ref_area = 1.0;        // Cl/Cd area: D for 2D (lbm.cpp:1402), pi D^2 / 4 for a sphere (lbm.cpp:3159)
    double body_radius = 0.0;     // IBM body radius (0: from the marker cloud)
    int thermal = 0;              // D3Q7 temperature population
    double tau_g = 0.0, T_ref = 0.0, gbeta[3] = {0, 0, 0};
    // ENERGY builds (-DENERGY): LBM.h's cp = k / (rho0 alpha) of the
    // viscous-heating source; tau_g above is its tau_g = 0.5 + alpha / cs2
    double cp = 0.0;
    // Rayleigh_Benard's MacroProp force F_y = g_beta (T - T_star) on every
    // cell (lbm.cpp:803-805), D3Q19 ENERGY builds; 0: the set-up force stays
    double g_beta = 0.0, T_star = 0.0;
    // Poiseuille_Flow builds: MacroProp sets the body force on every cell,
    // walls included (lbm.cpp:800-801); the body force itself is read from
    // fluid[..].F of the fluid cells at Init
    int wall_force = 0;
    int Nt = 10;                  // output cadence (LBM.h:493-496): Sup_MacroProp's told = (n - Nt) dt
    // OutputCSV's time column, (i + 1) csv_time_step: the reference's Nt dt
    // (Couette / Poiseuille / Rayleigh-Benard) or dt u_max / D (the IBM
    // cylinders) (lbm.cpp:3169-3186)
    double csv_time_step = 1.0;
    // Find_Nusselt_number's alpha and dT (LBM.h's Rayleigh_Benard block)
    double alpha = 0.0, dT = 1.0;
    // the reference's global centre (center_x, center_y, 1): IBLBM's box is
    // [centre - D, centre + D] (lbm.cpp:1165-1166); unset, the marker centroid
    int body_center_set = 0;
    double body_center[3] = {0, 0, 0};
    // D2Q9 IBLBM options (#define D2Q9 builds): the reference's nearest-node
    // density (lbm.cpp:1315-1317) and added mass (lbm.cpp:1392-1398, V_solid
    // = vsolid), the prescribed V_CM(t) (LBM_MOTION_*, lbm.cpp:1140-1151) and
    // the forcing scheme (0 implicit, 1 explicit)
    int rho_nearest = 0, added_mass = 0;
    double vsolid = 0.0;
    int motion = LBM_MOTION_FIXED;
    double motion_amp = 0.0, motion_freq = 0.0, motion_velocity[3] = {0, 0, 0};
    int ibm_scheme = 0;
};
extern lbm_options g_lbm_options;

class LATTICE {
  public:
    short type = TYPE_F;
    double density = 1.0;
    double ux = 0.0, uy = 0.0, uz = 0.0;
    double f[npop], f_star[npop];
    double F[3] = {0, 0, 0};
    double Fm[3] = {0, 0, 0};
    double T = 0.0;
#if defined ENERGY
    // LBM.h:590-596: the energy equation's populations stay on the device;
    // q (the heat flux sum g c) reaches the mirror with sync_to_host
    double g[npop], g_star[npop];
    double q[3] = {0, 0, 0};
    short type_Energy = TYPE_F;
    double F_vis[npop];
#endif
#if defined MORE_DETAILS
    // LBM.h:572-588; vorticity and its statistics stay zero, as in the
    // reference (whose vorticity code is commented out)
    double pressure = 0.0;
    double sigma[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double vorticity[3] = {0, 0, 0};
    double avg_velocity[3] = {0, 0, 0};
    double avg_pressure = 0;
    double avg_vorticity[3] = {0, 0, 0};
    double avg_ReynoldStress[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double rms_velocity[3] = {0, 0, 0};
    double rms_pressure = 0;
    double rms_vorticity[3] = {0, 0, 0};
    double rms_ReynoldStress[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#endif
};

class MARKER {
  public:
    double x, y, z = 1;
    double u_boundary[3] = {0, 0, 0};
    double u_boundary_des[3] = {0, 0, 0};
    double F_boundary[3] = {0, 0, 0};
    double normal[3] = {0, 0, 0};
    double Fm_boundary[3] = {0, 0, 0};
    // 2D normal t x z of the segment (x1,y1,z1)->(x2,y2,z2) (lbm.cpp:1048-1069)
    void Normal_Marker(int n, double x1, double x2, double y1, double y2, double z1, double z2);
};

struct lbm_device_state;  // shared by shallow copies of an LBM (the reference returns LBM by value)

class LBM {
  private:
    int Nx, Ny, Nz = 1;
    double tau;
    std::shared_ptr<lbm_device_state> dev;

  public:
    LATTICE ***fluid;

    LBM(int Nx, int Ny, int Nz, double tau);

    void Init();
    void Collision();
    void Streaming();
    void MacroProp();
    void ConvLBM(int i, int j, int k);          // host collision of one mirror cell (lbm.cpp:75-119)
    double Calc_feq(int i, int j, int k, int l); // third-order equilibrium (lbm.cpp:628-633)
    void Determine_Wall_Velocity(int i, int j, int k, std::vector<double> &uwall);  // lbm.cpp:941-962
#if defined ENERGY
    // ENERGY host helpers on the mirror (the device keeps g; the mirror's g
    // holds Init's equilibrium): Calc_geq (lbm.cpp:636-653), the wall T of
    // Determine_Wall_Temperature (lbm.cpp:965-981) and of
    // Determine_Twall_Neumann (lbm.cpp:983-1028), which also writes it into
    // the mirror's wall cell opposite the normal
    double Calc_geq(int i, int j, int k, int l, short type, std::vector<double> uwall);
    double Determine_Wall_Temperature(int i, int j, int k);
    double Determine_Twall_Neumann(int i, int j, int k, std::vector<double> uwall, std::vector<int> cdotn_pos,
                                   std::vector<int> cdotn_notpos, double j_dot_n);
#endif

    int getNx() const;
    int getNy() const;
    int getNz() const;
    double getTAU() const;

#if defined MORE_DETAILS
    // LBM::Sup_MacroProp (lbm.cpp:865-939) on the device; the statistics
    // reach fluid[..] with sync_to_host
    void Sup_MacroProp(int n);
#endif

    // GB300 additions
    void sync_to_host();        // MacroProp moments (MORE_DETAILS: and details, statistics) into fluid[..]
    lbm_handle *handle() const; // the device solve (nullptr before Init)
    lbm_energy3d *energy3d() const; // the D3Q19 ENERGY solve (-DENERGY without -DD2Q9 builds)
    long long steps() const;
    friend void IBLBM(LBM &lb, std::vector<MARKER> &marker, std::vector<double> &ds, std::vector<double> &Cl,
                      std::vector<double> &Cd, double V_CM[], double t);
};

void NearestLatticeCoordinate(int xmin, int xmax, int ymin, int ymax, int zmin, int zmax, int &i, int &j, int &k,
                              std::vector<MARKER> &marker, int n);
double kernel(double r);
double Calc_AverageDensity(LBM &lb, std::vector<MARKER> &marker, int xmin, int xmax, int ymin, int ymax, int zmin,
                           int zmax);
void IBLBM(LBM &lb, std::vector<MARKER> &marker, std::vector<double> &ds, std::vector<double> &Cl,
           std::vector<double> &Cd, double V_CM[], double t);
// Momentum-exchange lift / drag of the interior solid cells after the latest
// step (LBM.h:790-792); normalised with g_lbm_options u_max and ref_area.
double MEA_CL(LBM &lb, int xmin, int xmax, int ymin, int ymax, int zmin, int zmax);
double MEA_CD(LBM &lb, int xmin, int xmax, int ymin, int ymax, int zmin, int zmax);
// OutputVTK (LBM.h:776-846) from the device, written while the loop goes on;
// lbmgpu_output_wait(lb.handle()) finishes the file in flight.
void OutputVTK_async(int &nout, LBM &lb);
#if defined MORE_DETAILS
// OutputAVGVTK (LBM.h:780-782) from the device: ./avgfield.vtr
void OutputAVGVTK(int &nout, LBM &lb);
#endif
// The reference's output and analysis functions (LBM.h:770-835), same
// signatures: OutputVTK writes ./field%06d.vtr of the current state and
// returns once it is on disk; OutputVTK_Marker "wall_t <time / Nt>.vtk" of the
// markers on the device (or of the given vector before IBLBM registered
// them); OutputCSV "time,error" rows with g_lbm_options.csv_time_step;
// Find_Nusselt_number (lbmgpu_nusselt, with g_lbm_options alpha and dT) and
// Find_Maximum_uy of the current moments.
void OutputVTK(int &nout, LBM &lb);
void OutputVTK_Marker(int &time, std::vector<MARKER> &marker);
void OutputCSV(std::vector<double> &error, std::string name);
double Find_Nusselt_number(LBM &lb);
double Find_Maximum_uy(LBM &lb);
