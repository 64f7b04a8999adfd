/* ref_config.h -- compile-time configuration for the reference-literal
 * oracle build.  It is force-included (g++ -include) ahead of the reference
 * sources; it defines DEFINES_H, so the configuration block of the
 * reference's LBM.h (LBM.h:9-517) is skipped and these values are used
 * instead.  Everything after that block (lattice tables, LATTICE, LBM,
 * MARKER and all of lbm.cpp) is the reference's own code, unmodified.
 *
 * Two variants, chosen with -D:
 *   REF_CAVITY    D3Q19 box with ghost walls (the 3D lid-driven cavity).  The
 *                 Sphere_BB case flag is used only to select the reference's
 *                 3D code paths; the harness sets the geometry itself.
 *   REF_CYLINDER  D2Q9 implicit IBM cylinder (the shipped default case),
 *                 shrunk to test size; with REF_EXPLICIT the explicit
 *                 direct-forcing scheme instead.
 *   REF_TRANSVERSE  D2Q9 implicit IBM cylinder oscillating across the
 *                 stream (the reference's Cylinder_Transverse_Oscillation),
 *                 shrunk; REF_AMP and REF_FREQ set its amplitude and
 *                 frequency.
 *   REF_INLINE    D2Q9 implicit IBM cylinder oscillating along the stream
 *                 in fluid at rest (Cylinder_Inline_Oscillating, KC = 5),
 *                 REF_PERIOD steps per period.
 *   REF_ARBIE     D2Q9 implicit IBM cylinder towed at -u through fluid at
 *                 rest (Cylinder_IBM_Moving_Arbie), centre x = REF_CX.
 *   REF_POISEUILLE  D2Q9 body-forced channel (Poiseuille_Flow), Ny =
 *                 REF_NY, Re = REF_RE; with REF_ENERGY also the reference's
 *                 ENERGY model (walls at T = 1, viscous heating).
 *   REF_COUETTE   D2Q9 Couette flow with the reference's own thermal model
 *                 (ENERGY: temperature populations on the flow lattice,
 *                 viscous heating, Dirichlet walls), Ny = REF_NY, Re = REF_RE.
 *   REF_CYLBASIC  D2Q9 staircase cylinder with momentum-exchange Cl/Cd (the
 *                 reference's Cylinder_Basic case), REF_NX x REF_NY, REF_D,
 *                 REF_RE, REF_U.
 *   REF_TANDEM    D2Q9 staircase circles in tandem (Cylinder_Tandem_Circle),
 *                 REF_NB circles REF_LPD diameters apart; REF_TRIANGLE the
 *                 equilateral triangles of Cylinder_Tandem_Triangle.
 *   REF_RAYLEIGH  D3Q19 Rayleigh-Benard box with the reference's ENERGY model
 *                 (main_setup_RayleighBenard1): Dirichlet walls at y = 0 and
 *                 Ny + 1, Neumann walls elsewhere, the buoyancy of
 *                 MacroProp; REF_NX x REF_NY x REF_NZ, the constants of
 *                 LBM.h:222-242.
 *   REF_SPHERE    D3Q19 staircase sphere with momentum-exchange Cl/Cd (the
 *                 reference's Sphere_BB case), shrunk to test size; REF_D,
 *                 REF_RE and REF_U set the diameter, Reynolds number and
 *                 inflow velocity.
 * Sizes come from REF_NX/REF_NY/REF_NZ/REF_TAU (and REF_D, REF_NODES,
 * REF_MMAX for the cylinder).  REF_DETAILS (with REF_CAVITY) also switches on
 * the reference's MORE_DETAILS mode (LBM.h:55): pressure, viscous stress and
 * the Sup_MacroProp running averages.
 */
#include <cmath>
#include <iostream>
#include <string>
#include <vector>
using namespace std;

#define DEFINES_H

static const double PI = 3.14159265;  // LBM.h:74
#define rho0 1.0
#define dt 1.0
#define dx 1.0
#define dy 1.0
#define dz 1.0
static const double cs2 = pow(dx, 2) / (3 * pow(dt, 2));
#define p0 rho0 *cs2
#define Conventional_LBM

#if defined REF_DETAILS
#define MORE_DETAILS
#endif

#define TYPE_F 0
#define TYPE_S 1
#define TYPE_OUT 2
#define TYPE_IN 3
#define TYPE_P 4
#define TYPE_L 5
#define TYPE_T 6
#define TYPE_Q 7

#if defined REF_CAVITY
#define Sphere_BB
#define MOMENTUM_EXCHANGE_ALGORITHM
#define D3Q19
#define Re 200.0
static const double D = 20;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = REF_NZ;
static const double u_max = 0.1;
static double center_x = dx * (Nx / 5.0);
static double center_y = dy * (Ny / 2.0);
static double center_z = dz * (Nz / 2.0);
static const double tau = REF_TAU;
static const double nu = cs2 * (tau - 0.5);
#define T_OUT 30000
#define Nt 10
#elif defined REF_CYLINDER
#define IBM
#if defined REF_EXPLICIT
#define Explicit_Diffuse_Interface_Scheme
#else
#define Implicit_Diffuse_Interface_Scheme
#endif
#define Cylinder_IBM
#define Volume_Force
#define D2Q9
#define Re 40.0
static const double D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static const double u_max = 0.1;
static double center_x = dx * (Nx / 5.0);
static double center_y = dy * (Ny / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
static const int number_nodes = REF_NODES;
static const int level_marker = 1;
static int m_max = REF_MMAX;
static const double Vsolid = PI * D * D * 0.25;
#define T_OUT 30000
#define Nt 10
#elif defined REF_TRANSVERSE
#define IBM
#define Implicit_Diffuse_Interface_Scheme
#define Cylinder_Transverse_Oscillation
#define Volume_Force
#define D2Q9
#define Re 100.0
static const double D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static const double u_max = 0.05;
static const double amplitude = REF_AMP;
static const double frequency_e = REF_FREQ;
// the quantities the reference derives frequency_e from (LBM.h:407-414),
// printed by print_Info only
static const double ratio_Amd = amplitude / D;
static const double frequency_ratio = 1.2;
static const double frequency_0 = frequency_e / frequency_ratio;
static const double Strouhal_number = frequency_0 * D / u_max;
static double center_x = dx * (Nx / 5.0);
static double center_y = dy * (Ny / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
static const double Vsolid = PI * D * D * 0.25 * (Nz + 2);
static const int number_nodes = REF_NODES;
static const int level_marker = 1;
static int m_max = REF_MMAX;
#define T_OUT 30000
#define Nt 10
#elif defined REF_INLINE
#define IBM
#define Implicit_Diffuse_Interface_Scheme
#define Cylinder_Inline_Oscillating
#define Volume_Force
#define D2Q9
#define Re 100.0
#define KC 5.0
static const double D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static const double period = REF_PERIOD;
static const double frequency = 1 / period;
static const double u_max = KC * D * frequency;
static const double amplitude = u_max / (2 * PI * frequency);
static double center_x = dx * (Nx / 2.0);
static double center_y = dy * (Ny / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
static const double Vsolid = PI * D * D * 0.25 * (Nz + 2);
static const int number_nodes = REF_NODES;
static const int level_marker = 1;
static int m_max = REF_MMAX;
#define T_OUT 30000
#define Nt 10
#elif defined REF_ARBIE
#define IBM
#define Implicit_Diffuse_Interface_Scheme
#define Cylinder_IBM_Moving_Arbie
#define Volume_Force
#define D2Q9
#define Re 40.0
static const double D = REF_D;
static const double target_tstar = 50;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static const double u_max = 0.1;
static double center_x = REF_CX;
static double center_y = dy * (Ny / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
static const int number_nodes = REF_NODES;
static const int level_marker = 1;
static int m_max = REF_MMAX;
static const double Vsolid = PI * D * D * 0.25;
#define T_OUT 30000
#define Nt 10
#elif defined REF_POISEUILLE
#define Poiseuille_Flow
#define D2Q9
#if defined REF_ENERGY
#define ENERGY
#endif
#define Re REF_RE
static const int Nx = 2;
static const int Ny = REF_NY;
static const int Nz = 2;
static const double tau = 0.9;
static const double nu = cs2 * (tau - 0.5);
static const double u_max = Re * nu / (Ny + 1);
static double dp_dx = -8 * rho0 * nu * u_max / pow(Ny + 1, 2);
#define Velocity_Ratio
#define Temperature_Ratio
static const double Pr = 0.7;
static const double alpha = nu / Pr;
static const double tau_g = 0.5 + alpha / (cs2 * dx);
static const double k = cs2 * tau_g * dx;
static const double cp = k / (rho0 * alpha);
static const double Tt = 1;
static const double Tb = 1;
static const double dT = 1;
static const double j_dot_n = 0;
static const double D = 1;
#define T_OUT 30000
#define Nt 10
#elif defined REF_COUETTE
#define Couette_Flow
#define ENERGY
#define D2Q9
#define Re REF_RE
static const int Nx = 2;
static const int Ny = REF_NY;
static const int Nz = 2;
static const double tau = 0.9;
static const double nu = cs2 * (tau - 0.5);
static const double u_wall = Re * nu / (Ny + 1);
static const double u_max = u_wall;
static double uwall_topx = u_wall;
static double uwall_botx = 0;
#define Velocity_Ratio
#define Temperature_Ratio
static const double Pr = 0.7;
static const double Br = 10;
static const double Ec = Br / Pr;
static const double alpha = nu / Pr;
static const double tau_g = 0.5 + alpha / (cs2 * dx);
static const double k = cs2 * tau_g * dx;
static const double cp = k / (rho0 * alpha);
static const double Tb = 0.5;
static const double dT = pow(u_wall, 2) / (cp * Ec);
static const double Tt = Tb + dT;
static const double j_dot_n = 0;
static const double D = 1;
#define T_OUT 30000
#define Nt 10
#elif defined REF_RAYLEIGH
#define Rayleigh_Benard
#define ENERGY
#define D3Q19
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = REF_NZ;
static const double Tb = 2;
static const double dT = 1;
static const double Tt = Tb - dT;
static const double j_dot_n = 0;
static const double Ra = 1710;
static const double g_beta = pow(10, -5);
static const double Pr = 0.71;
static const double nu = sqrt(g_beta * dT * pow(Nz + 1, 3) * Pr / Ra);
static const double tau = 0.5 + nu / cs2;
static const double alpha = nu / Pr;
static const double tau_g = 0.5 + alpha / (cs2 * dx);
static const double k = cs2 * tau_g * dx;
static const double cp = k / (rho0 * alpha);
// not in the reference's Rayleigh_Benard block, which therefore does not
// compile as shipped: OutputVTK (lbm.cpp:2446) scales u by it; the harness
// never calls the writer
static const double u_max = 1.0;
#define T_OUT 30000
#define Nt 10
#elif defined REF_SPHERE
#define Sphere_BB
#define MOMENTUM_EXCHANGE_ALGORITHM
#define D3Q19
#define Re REF_RE
static const double D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = REF_NZ;
static const double u_max = REF_U;
static double center_x = dx * (Nx / 5.0);
static double center_y = dy * (Ny / 2.0);
static double center_z = dz * (Nz / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
#define T_OUT 30000
#define Nt 10
#elif defined REF_CYLBASIC
#define Cylinder_Basic
#define MOMENTUM_EXCHANGE_ALGORITHM
#define D2Q9
#define Re REF_RE
static const double D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static const double u_max = REF_U;
static double center_x = dx * (Nx / 5.0);
static double center_y = dy * (Ny / 2.0);
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
#define T_OUT 30000
#define Nt 10
#elif defined REF_TANDEM
#define Cylinder_Tandem_Circle
#define MOMENTUM_EXCHANGE_ALGORITHM
#define D2Q9
#define Re REF_RE
static int D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static double LpD = REF_LPD;
static double L = D * LpD;
static int N = REF_NB;
static int center_x = Nx / 5;
static int center_y = Ny / 2 + L / 2;
static double u_max = REF_U;
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
#define T_OUT 30000
#define Nt 10
#elif defined REF_TRIANGLE
#define Cylinder_Tandem_Triangle
#define MOMENTUM_EXCHANGE_ALGORITHM
#define D2Q9
#define Re REF_RE
static int D = REF_D;
static const int Nx = REF_NX;
static const int Ny = REF_NY;
static const int Nz = 1;
static double LpD = REF_LPD;
static int N = REF_NB;
static int tip_x = Nx / 5;
static int tip_y = Ny / 2;
static double L = D * LpD;
static double u_max = REF_U;
static const double nu = u_max * D / Re;
static const double tau = 0.5 * dt + nu / cs2;
#define T_OUT 30000
#define Nt 10
#else
#error "define one of the REF_* variants listed above"
#endif
