/*
 * lbmgpu.h -- C ABI of the GB300 LBM time-step library (liblbmgpu.so).
 *
 * Plain C types only (no CUDA or torch types).  The entry points replace the
 * hot path of the reference's LBM class and IBM driver
 * (DestinyFlow01/Lattice-Boltzmann-Method---Graduate-FSI-):
 *
 *   reference                                   here
 *   LBM::LBM(Nx,Ny,Nz,tau)        LBM.h:630    lbmgpu_config_from_types + lbmgpu_create
 *   fluid[i][j][k].type / ux..    LBM.h:558-597 (geometry)  lbmgpu_config_from_types
 *   LBM::Init                     lbm.cpp:31   lbmgpu_init / lbmgpu_init_fields
 *   LBM::Collision + Streaming    lbm.cpp:60,182  lbmgpu_step (fused)
 *   LBM::MacroProp                lbm.cpp:657  fused into lbmgpu_step; read back
 *                                              with lbmgpu_download
 *   IBLBM (markers, ds, Cl, Cd)   lbm.cpp:1135 lbmgpu_set_markers (+ forcing inside
 *                                              lbmgpu_step), lbmgpu_get_forces
 *   terminate() on bad state      lbm.cpp:116,774  lbmgpu_status (never aborts)
 *
 * Conventions.  Interior cells only on the device; host arrays passed to or
 * returned by the ABI are x-fastest: index i + nx*(j + ny*k) for interior
 * cell (i+1, j+1, k+1) of the reference's fluid[Nx+2][Ny+2][Nz+2] array.
 * Geometry arrays given to lbmgpu_config_from_types include the ghost layers:
 * index i + (nx+2)*(j + (ny+2)*k) for fluid[i][j][k].
 *
 * Every call returns an lbm_status; lbmgpu_last_error() gives a message for
 * the calling thread.  A handle owns one CUDA stream; calls on one handle are
 * not re-entrant, distinct handles are independent.
 */
#ifndef LBMGPU_H
#define LBMGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lbm_status {
    LBM_OK = 0,
    LBM_ERR_INVALID = 1,     /* bad argument or configuration */
    LBM_ERR_CUDA = 2,        /* CUDA runtime error */
    LBM_ERR_NOMEM = 3,       /* device or host allocation failed */
    LBM_ERR_DIVERGED = 4,    /* device status word reports an invalid state */
    LBM_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
    LBM_ERR_STATE = 6,       /* call out of order (e.g. step before init) */
    LBM_ERR_UNSUPPORTED = 7  /* a set-up or option the library does not handle */
} lbm_status;

/* Population storage formats.  F16/BF16 store f - w (shifted) and compute in FP32. */
enum { LBM_STORE_F32 = 0, LBM_STORE_F16 = 1, LBM_STORE_BF16 = 2 };

/* Kind of one box face (its ghost layer).  Reference cell types (LBM.h:505-515):
 * TYPE_S -> WALL, TYPE_IN -> INLET, TYPE_OUT -> OUTLET_EQ (populations from the
 * ghost keep the initial equilibrium, as in the reference), TYPE_F ghost layers
 * on both faces of an axis -> PERIODIC.  OUTLET_ZG (zero-gradient) is new. */
enum { LBM_FACE_WALL = 0, LBM_FACE_INLET = 1, LBM_FACE_OUTLET_EQ = 2, LBM_FACE_OUTLET_ZG = 3, LBM_FACE_PERIODIC = 4 };

/* Thermal condition on a WALL face. */
/* Thermal wall kinds.  NEUMANN (D2Q9 ENERGY handles only): the wall's T is
 * set every streaming so that no heat crosses it, j . n = 0 (the reference's
 * j_dot_n; Determine_Twall_Neumann, lbm.cpp:983-1028).  ADIABATIC on ENERGY
 * handles: the wall's links are never streamed and keep their initial
 * values, as a wall of any other type_Energy in the reference
 * (lbm.cpp:276-288).  On ENERGY handles every wall face's T is its set-up
 * temperature: the Dirichlet walls' temperature is the mean of their solid
 * neighbours' (lbm.cpp:965-981), which wraps onto the opposite wall row. */
enum { LBM_TWALL_ADIABATIC = 0, LBM_TWALL_DIRICHLET = 1, LBM_TWALL_NEUMANN = 2 };

/* Fields for lbmgpu_download*. */
enum { LBM_FIELD_RHO = 0, LBM_FIELD_UX = 1, LBM_FIELD_UY = 2, LBM_FIELD_UZ = 3, LBM_FIELD_T = 4,
       /* heat flux sum g c (lbm.cpp:778-792), thermal solves */
       LBM_FIELD_QX = 5, LBM_FIELD_QY = 6, LBM_FIELD_QZ = 7 };

/* Device status bits (lbmgpu_status). */
enum {
    LBM_STATUS_RHO_RANGE = 1,   /* rho outside (0, 100) or NaN: lbm.cpp:772-775 */
    LBM_STATUS_BAND_EDGE = 2,   /* an IBM stencil reached outside the band/interior */
    LBM_STATUS_NONFINITE_FORCE = 4,
    LBM_STATUS_TIMEOUT = 16,    /* a bounded device wait (mbarrier, grid barrier) gave up */
    LBM_STATUS_T_RANGE = 32     /* ENERGY: T outside (0, 100) or NaN: lbm.cpp:794-797 */
};

typedef struct lbm_face {
    int kind;          /* LBM_FACE_* */
    int thermal_kind;  /* LBM_TWALL_* for walls */
    double rho;        /* inlet/outlet-equilibrium density */
    double u[3];       /* wall velocity, or inlet/outlet-equilibrium velocity */
    double T;          /* inlet temperature or (set-up) wall temperature */
} lbm_face;

typedef struct lbm_config {
    int nx, ny, nz;       /* interior cells (Nx, Ny, Nz) */
    double tau;           /* BGK relaxation time */
    int storage;          /* LBM_STORE_* */
    lbm_face faces[6];    /* x-, x+, y-, y+, z-, z+ */
    double rho0;          /* uniform initial density (lbmgpu_init) */
    double u0[3];         /* uniform initial velocity */
    double body_force[3]; /* uniform body force (e.g. -dp/dx, lbm.cpp:800-801) */
    int thermal;          /* 1: D3Q7 temperature population */
    double tau_g;         /* thermal relaxation time, 0.5 + alpha / (1/4) */
    double T_init;        /* uniform initial temperature */
    double T_ref;         /* Boussinesq reference temperature T0 */
    double gbeta[3];      /* Boussinesq: F += gbeta * (T - T0)  (lbm.cpp:804-805) */
    int block_x, block_y; /* thread-block shape of the fused kernel; 0 = default */
    int graph_steps;      /* steps per captured CUDA graph; 0 = default, <0 = no graphs */
    int staged;           /* must be 0: reserved (a tensor-copy staged step kernel, removed after it measured
                             slower than direct loads in every variant) */
    int ibm_overlap;      /* 0: a fixed body's IBM phase overlaps the far-region streaming (second
                             stream; D3Q19 and D2Q9); <0: serial */
    int xface;            /* 0: lanes on x = 0 / x = nx-1 keep the plain pull and redo their five
                             x-crossing links; <0: their whole warp takes the boundary-class path */
    int lattice;          /* LBM_LATTICE_*: 0 or 19 = D3Q19; 9 = D2Q9 (the reference's #define D2Q9
                             build; nz = 1, faces 4/5 unused) */
    double cp;            /* thermal == LBM_THERMAL_ENERGY: specific heat capacity of the viscous-heating
                             source Phi / cp (LBM.h:213) */
    int wall_force;       /* D2Q9: 1 = the body force also acts on the wall cells, as the reference's
                             Poiseuille_Flow MacroProp sets it on every cell (lbm.cpp:800-801); the walls
                             then report u_w + F/2 and bounce back as moving walls from the third
                             streaming on */
    int cells_per_thread; /* D3Q19 fused step: consecutive x-cells per thread, moved as one 4-, 8- or
                             16-byte access per population row and updated in pairs with the packed FP32
                             instructions (FP16/BF16: 2, 4 or 8; FP32: 2 or 4); 0 = default (2 for
                             FP16/BF16 on lattices of 2^20 cells or more, else 1); 1 = one cell per
                             thread.  Needs nx a multiple of it, else one cell per thread is used.
                             Results are identical either way. */
} lbm_config;

/* lbm_config.thermal: 0 none; 1 a D3Q7 temperature population with a heat
 * source and Boussinesq buoyancy (D3Q19 handles); 2 the reference's own
 * ENERGY model (LBM.h:58): temperature populations on the flow lattice with
 * the cubic equilibrium, viscous heating, and Dirichlet, Neumann or adiabatic
 * walls (D2Q9 handles; faces periodic or walls).  The ENERGY model on D3Q19
 * is a solver object of its own: lbmgpu_energy3d_create. */
enum { LBM_THERMAL_NONE = 0, LBM_THERMAL_D3Q7 = 1, LBM_THERMAL_ENERGY = 2 };

enum { LBM_LATTICE_D3Q19 = 19, LBM_LATTICE_D2Q9 = 9 };

/* Prescribed body velocity V_CM(t) of a two-dimensional IBM body (IBLBM,
 * lbm.cpp:1140-1151), t = step * dt: FIXED 0 (Cylinder_IBM); CONSTANT the
 * lbm_ibm_config velocity (Cylinder_IBM_Moving_Arbie); INLINE_OSC
 * V_x = -amp cos(2 pi f t) (Cylinder_Inline_Oscillating); TRANSVERSE_OSC
 * V_y = -2 pi f amp sin(2 pi f t) (Cylinder_Transverse_Oscillation). */
enum { LBM_MOTION_FIXED = 0, LBM_MOTION_CONSTANT = 1, LBM_MOTION_INLINE_OSC = 2, LBM_MOTION_TRANSVERSE_OSC = 3 };

typedef struct lbm_ibm_config {
    int n_markers;
    int m_max;            /* implicit forcing iterations (lbm.cpp:1311) */
    int literal_sign;     /* 1: force -Fm but velocity +Fm/2rho (lbm.cpp:1347-1352) */
    int free_body;        /* 0: fixed/prescribed, 1: FP64 Newton-Euler (Kempe-Froehlich internal fluid) */
    int thermal;          /* 1: also force the temperature to T_body */
    double radius;        /* body radius (band size and rigid body) */
    double center[3];     /* body centre, reference node coordinates */
    double density_ratio; /* rho_s / rho_f */
    double volume;        /* V_s */
    double inertia;       /* I_p = 2/5 rho_s V_s R^2 for a sphere */
    double gravity[3];
    double velocity[3];   /* initial body velocity */
    double T_body;        /* marker temperature for the thermal IBM */
    int free_dofs;        /* free body: bits 0-2 translation x,y,z, bits 3-5 rotation; 0 = all six */
    /* D2Q9 handles: the options of the reference's two-dimensional IBLBM */
    int rho_nearest;      /* 1: marker density at NearestLatticeCoordinate over the whole box
                             (lbm.cpp:1315-1317; needs normals); 0: delta-interpolated */
    int added_mass;       /* 1: Drag/Lift += rho_avg V_s (V - V_before) / dt with rho_avg of
                             Calc_AverageDensity (lbm.cpp:1105-1132, 1392-1398; needs normals) */
    int motion;           /* LBM_MOTION_* */
    double motion_amp, motion_freq;
    int scheme;           /* 0: implicit multi-direct forcing (lbm.cpp:1259-1390);
                             1: explicit direct forcing (lbm.cpp:1171-1258) */
    double virtual_mass;  /* free body: virtual-mass coefficient C_v of Schwarz, Kempe & Froehlich (2015);
                             0 = plain explicit Newton-Euler; 1 keeps light bodies (rho_s/rho_f ~ 1.5)
                             stable in rotation and translation */
} lbm_ibm_config;

typedef struct lbm_handle lbm_handle;

/* Derive a configuration from the reference's per-cell description
 * (fluid[i][j][k].type and the ghost velocities/densities/temperatures),
 * arrays of (nx+2)(ny+2)(nz+2) entries, x fastest; u/rho/T may be NULL.
 * Interior TYPE_S cells at rest are accepted: pass their mask to
 * lbmgpu_set_solids.  Fails with LBM_ERR_UNSUPPORTED for other non-fluid
 * interior cells, moving interior solids, or a face that is not uniform.
 * Periodic axes (TYPE_F ghost layers) are mapped to an interior of N+2
 * cells, as the reference wraps over N+2 (lbm.cpp:187-189). */
lbm_status lbmgpu_config_from_types(int nx, int ny, int nz, double tau, const uint8_t *types, const double *rho,
                                    const double *ux, const double *uy, const double *uz, const double *T,
                                    lbm_config *out);

/* The same for the reference's D2Q9 build (Nz = 1): arrays of (nx+2)(ny+2)
 * entries, x fastest, the computational layer fluid[i][j][1].  The result
 * has lattice = LBM_LATTICE_D2Q9 and nz = 1.  Interior TYPE_S cells at rest
 * are accepted: pass their mask to lbmgpu_set_solids. */
lbm_status lbmgpu_config_from_types_2d(int nx, int ny, double tau, const uint8_t *types, const double *rho,
                                       const double *ux, const double *uy, lbm_config *out);

/* Adds the reference's ENERGY model to a D2Q9 configuration made by
 * lbmgpu_config_from_types_2d from the same (nx+2)(ny+2) arrays: the
 * type_Energy of the ghost cells (TYPE_T = 6 on every wall cell: Dirichlet,
 * lbm.cpp:277-280) and the set-up temperature T, ghosts included (uniform on
 * each wall face and over the fluid).  tau_g and cp are LBM.h's
 * tau_g = 0.5 + alpha / cs2 and cp = k / (rho0 alpha).  Replaces the
 * LATTICE::type_Energy / T set-up of main_setup_Couette (lbm.cpp:1552-1572).
 * type_Energy TYPE_Q (7) makes a Neumann face, any other type an adiabatic
 * one (LBM_TWALL_*).  Fails with LBM_ERR_UNSUPPORTED for inlet/outlet faces,
 * a face mixing thermal wall types, or a non-uniform set-up. */
lbm_status lbmgpu_config_energy_2d(lbm_config *cfg, int nx, int ny, const uint8_t *types, const uint8_t *types_energy,
                                   const double *T, double tau_g, double cp);

lbm_status lbmgpu_create(const lbm_config *cfg, lbm_handle **out);
lbm_status lbmgpu_destroy(lbm_handle *h);

/* LBM::Init (lbm.cpp:31-57): f = feq(rho0, u0) (third order), g = geq(T_init). */
lbm_status lbmgpu_init(lbm_handle *h);
/* LBM::Init from per-cell fields (interior, x fastest); T may be NULL. */
lbm_status lbmgpu_init_fields(lbm_handle *h, const double *rho, const double *ux, const double *uy, const double *uz,
                              const double *T);

/* IBLBM set-up (lbm.cpp:1135-1167): markers xyz ([3][n], reference node
 * coordinates), weights ds ([n]), desired velocities udes ([3][n], NULL =
 * the body velocity). */
lbm_status lbmgpu_set_markers(lbm_handle *h, const lbm_ibm_config *ic, const double *xyz, const double *ds,
                              const double *udes);
/* Outward marker normals ([3][n], MARKER::normal, lbm.cpp:1048-1069) for
 * the nearest-node density and the added-mass average of a D2Q9 handle;
 * call after lbmgpu_set_markers. */
lbm_status lbmgpu_set_marker_normals(lbm_handle *h, const double *nxyz);

/* Advance n reference iterations (IBLBM -> Collision -> Streaming, or
 * Collision -> Streaming -> MacroProp).  Asynchronous on the handle's stream. */
lbm_status lbmgpu_step(lbm_handle *h, int nsteps);

/* lbmgpu_step bracketed by CUDA events on the handle's stream (graph replay
 * included): device time of the n steps. */
lbm_status lbmgpu_step_timed(lbm_handle *h, int nsteps, double *ms);

/* Steps launched one by one with CUDA events on the handle's stream: total
 * device time of the n steps and the summed device time of the fused
 * collide-stream kernel. */
lbm_status lbmgpu_step_profiled(lbm_handle *h, int nsteps, double *total_ms, double *fused_ms);

/* As lbmgpu_step_profiled, split further: phases[0] total, [1] fused
 * collide-stream launches (far + near), [2] the near-region launch alone,
 * [3] the IBM phase (interpolation/spreading, band collision, reductions),
 * each summed over the n steps, in milliseconds.  With the IBM phase
 * overlapped, [3] runs concurrently with the next step's far launch. */
lbm_status lbmgpu_step_phases(lbm_handle *h, int nsteps, double *phases);

/* MacroProp moments of the current state (rho, u = (sum f c + F/2)/rho, T),
 * interior cells, x fastest. */
lbm_status lbmgpu_download(lbm_handle *h, int field, double *host);
lbm_status lbmgpu_download_f32(lbm_handle *h, int field, float *host);
/* All of rho, ux, uy, uz (and T if thermal) in one export, FP32, [field][cells]. */
lbm_status lbmgpu_download_all_f32(lbm_handle *h, float *host);
/* The same read-back without waiting: the moment export runs on the handle's
 * stream and the copy to `host` (pinned memory, e.g. lbmgpu_host_alloc, for
 * a true overlap) on a copy stream of its own, so the steps enqueued next
 * run while it lands.  The data are in `host` after lbmgpu_download_wait or
 * lbmgpu_sync.  A later export waits for this copy before it rewrites the
 * device moments.  D2Q9 handles copy synchronously. */
lbm_status lbmgpu_download_all_f32_async(lbm_handle *h, float *host);
lbm_status lbmgpu_download_wait(lbm_handle *h);

/* IBM force history, oldest first: per step {Fx, Fy, Fz, Tx, Ty, Tz, heat,
 * step}, where F = sum over forcing iterations of -F_m ds_m (the reference's
 * Drag/Lift accumulators, lbm.cpp:1322-1323).  *n_out = entries written. */
/* Interior solid cells at rest -- staircase bodies such as the reference's
 * Generate_Sphere (lbm.cpp:1759-1787) or its cylinders: mask has nx*ny*nz
 * entries (x fastest), non-zero = TYPE_S.  Their links bounce back (halfway,
 * lbm.cpp:252-274) inside the fused step and the momentum exchange on them is
 * recorded every step.  Call after lbmgpu_create and before lbmgpu_init; a
 * fixed IBM body on the same handle then keeps the serial order. */
lbm_status lbmgpu_set_solids(lbm_handle *h, const uint8_t *mask);

/* Momentum exchange on the solid cells, MEA_CD / MEA_CL (lbm.cpp:3085-3163)
 * summed over every fluid cell next to a solid: rows of 4 doubles
 * (Fx, Fy, Fz, step) for reference steps 1 .. n (the last max_steps of
 * them), F = -sum (f*_l + f_opp(l)) c_l in lattice units.  The reference's
 * coefficients are Cd = Fx / (0.5 rho0 U^2 A), Cl = -Fy / (0.5 rho0 U^2 A). */
lbm_status lbmgpu_get_solid_forces(lbm_handle *h, double *out, int max_steps, int *n_out);

/* Momentum exchange over one box of the current state, MEA_CL / MEA_CD
 * (lbm.cpp:3085-3163) called after a step: box = (xmin, xmax, ymin, ymax,
 * zmin, zmax) in the reference's ghost-inclusive indices, inclusive, as its
 * callers pass them (main.cpp:246-353).  out = F = -sum (f*_l + f_opp(l)) c_l
 * over the fluid cells of the box and their solid links; Cd = Fx / q,
 * Cl = -Fy / q.  D2Q9 handles (several bodies, one box each: the tandem
 * cases); a D3Q19 handle returns LBM_ERR_UNSUPPORTED (its
 * lbmgpu_get_solid_forces sums every solid after every step). */
lbm_status lbmgpu_mea_box(lbm_handle *h, const int box[6], double out[3]);

/* Find_Nusselt_number (lbm.cpp:3538-3561) of the current state:
 * Nu = 1 + <u_y T> / (alpha dT / (Ny + 1)), the mean over the fluid cells
 * (interior solids excluded), Ny the reference's interior row count.  Thermal
 * handles: D3Q7 (D3Q19) or ENERGY (D2Q9).  The reference also counts
 * TYPE_IN / TYPE_OUT ghost cells, which are not on the device; for closed or
 * periodic boxes (its Rayleigh-Benard, Couette and Poiseuille cases) the set
 * of cells is the same.  Summed in FP64 in a fixed order. */
lbm_status lbmgpu_nusselt(lbm_handle *h, double alpha, double dT, double *out);

/* The IBM body's force rows of the last min(steps done, 65536, max_steps)
 * steps, oldest first, 8 doubles a row into out; *n_out = the rows written.
 * D3Q19: the FP64 sums over the markers of -F_m ds_m (x, y, z), their torque
 * about the body centre (x, y, z), the heat exchange, and the step's index
 * (the steps done before it).  D2Q9: drag and lift (IBLBM's sums,
 * lbm.cpp:1392-1416, with the added-mass term when set), five zeros, and the
 * reference's 1-based step.  Cl/Cd = row / (0.5 u^2 area).  One kernel copies
 * the rows into pinned, device-mapped host memory; the call synchronises the
 * handle's stream once. */
lbm_status lbmgpu_get_forces(lbm_handle *h, double *out, int max_steps, int *n_out);

/* New positions (3 x n, x rows first) and weights (n) for the markers that
 * lbmgpu_set_markers registered, as the caller moves the body between calls
 * of IBLBM (its marker array is an input of every call, lbm.cpp:1135-1167).
 * The copies are enqueued on the handle's stream ahead of the next step and
 * nothing else is reset, so captured graphs stay valid; keep the host arrays
 * (pinned memory for a true overlap) unchanged until the next synchronising
 * call.  The markers must stay inside the band set up by lbmgpu_set_markers
 * (LBM_STATUS_BAND_EDGE otherwise).  D3Q19 handles. */
lbm_status lbmgpu_update_markers(lbm_handle *h, const double *xyz, const double *ds);

/* Checkpoint and restart (no counterpart in the reference, which restarts
 * from its set-up): the current populations, the device state (step counters,
 * band origin, rigid body), the markers and the force histories.  Load onto a
 * handle created with the same configuration and the same lbmgpu_set_markers /
 * lbmgpu_set_solids (D2Q9: lbmgpu_set_marker_normals) calls, instead of
 * lbmgpu_init; the run then continues as if never interrupted, bit for bit.
 * D3Q19 and D2Q9 handles (each its own file format). */
lbm_status lbmgpu_save_state(lbm_handle *h, const char *path);
lbm_status lbmgpu_load_state(lbm_handle *h, const char *path);

/* ------------------------------------------------------------------------
 * MORE_DETAILS mode (LBM.h:55): pressure, viscous stress and the running
 * statistics of Sup_MacroProp.  A run-time switch per handle here.
 * ---------------------------------------------------------------------- */

/* Components of lbmgpu_download_details ([7][cells], FP32): MacroProp's
 * pressure = rho / 3 and viscous stress
 * sigma_ab = -(tau - 1/2) / tau * sum_l f_l (c_la - u_a)(c_lb - u_b)
 * (lbm.cpp:681-705) of the current state; sigma is symmetric, its six
 * distinct components are given. */
enum { LBM_DETAIL_P = 0, LBM_DETAIL_SXX = 1, LBM_DETAIL_SXY = 2, LBM_DETAIL_SXZ = 3, LBM_DETAIL_SYY = 4,
       LBM_DETAIL_SYZ = 5, LBM_DETAIL_SZZ = 6, LBM_DETAIL_COUNT = 7 };

/* Components of lbmgpu_download_stats ([20][cells], FP64): the
 * Sup_MacroProp averages and rms values (lbm.cpp:865-939) of velocity (3),
 * pressure (1) and Reynolds stress (6 distinct: xx xy xz yy yz zz).  The
 * reference never computes the vorticity (lbm.cpp:712-770 is commented out):
 * its averages and rms values are zero and not held. */
enum { LBM_STAT_AVG_U = 0, LBM_STAT_AVG_P = 3, LBM_STAT_AVG_RS = 4, LBM_STAT_RMS_U = 10, LBM_STAT_RMS_P = 13,
       LBM_STAT_RMS_RS = 14, LBM_STAT_COUNT = 20 };

/* on = 1: allocate the detail and statistics arrays (7 floats + 20 doubles
 * per cell), clear the statistics, and add the Pressure / Viscous Stress /
 * Vorticity arrays of the reference's MORE_DETAILS OutputVTK to
 * lbmgpu_output_vtk_async.  on = 0 frees them.  D2Q9 handles too (their
 * z components are zero), except those with markers: the reference's IBM
 * loop never calls MacroProp, which forms the details (LBM_ERR_UNSUPPORTED,
 * in either order of this call and lbmgpu_set_markers). */
lbm_status lbmgpu_set_more_details(lbm_handle *h, int on);
/* Pressure and viscous stress of the current state, [LBM_DETAIL_COUNT][cells]. */
lbm_status lbmgpu_download_details(lbm_handle *h, float *host);
/* LBM::Sup_MacroProp(n) (lbm.cpp:865-939; main.cpp:389 calls it every Nt
 * steps): fold the current state into the statistics with
 * told = (n - nt) * dt, the reference's weights included (the velocity
 * sample weighted dt, the others 1; the pressure rms squares the current
 * pressure, lbm.cpp:913).  Synchronous. */
lbm_status lbmgpu_sup_macroprop(lbm_handle *h, int n, int nt, double dt);
/* The statistics, [LBM_STAT_COUNT][cells]; samples / told (may be NULL): how
 * many samples were folded in and the told of the latest one. */
lbm_status lbmgpu_download_stats(lbm_handle *h, double *host, int *samples, double *told);

/* ------------------------------------------------------------------------
 * Output in the reference's file formats.
 * ---------------------------------------------------------------------- */

/* OutputVTK (lbm.cpp:2290-2642): a RectilinearGrid .vtr of the current state
 * -- Density, Velocity / u_ref, Force density (IBM), Temperature and Heat flux
 * (thermal), CellType -- over the reference's cells i = 0..Nx+1,
 * j = 0..Ny+1, k = 1..Nz, appended raw Float32 data.  Ghost cells carry their
 * face's boundary state (a moving wall at edges).  types: the ghost-inclusive
 * fluid[..].type array given to lbmgpu_config_from_types, for the CellType
 * array (NULL: derived from the faces and the solid mask).  Returns once the
 * snapshot is enqueued; a host thread writes the file while the device goes
 * on stepping.  One file is in flight at a time: the next call (or
 * lbmgpu_output_wait) finishes the previous one and returns its status.
 * D2Q9 handles (the reference's #define D2Q9 build) write the layer k = 1 of
 * fluid[Nx+2][Ny+2][3]: types is then that (Nx+2)(Ny+2) layer; the moments are
 * copied out before the call returns, and an IBM body's Force density is the
 * force its box cells collided with (IBLBM's fluid[..].F). */
lbm_status lbmgpu_output_vtk_async(lbm_handle *h, const char *path, double u_ref, const uint8_t *types);
lbm_status lbmgpu_output_wait(lbm_handle *h);

/* OutputAVGVTK (lbm.cpp:2644-3031), MORE_DETAILS mode: Density, Velocity,
 * Avg / Rms velocity (/ u_ref), Pressure, Avg / Rms pressure, Viscous Stress,
 * Vorticity, Avg / Rms vorticity (zero, as in the reference), Avg / Rms
 * Reynolds stress (/ u_ref^2), CellType; ghost cells carry the statistics a
 * cell held at its face's state since the first sample.  Synchronous. */
lbm_status lbmgpu_output_avg_vtk(lbm_handle *h, const char *path, double u_ref, const uint8_t *types);

/* OutputVTK_Marker (lbm.cpp:3033-3077): legacy ASCII POLYDATA of the markers
 * (points, closed polyline, vertices); D3Q19 and D2Q9 handles. */
lbm_status lbmgpu_output_markers_vtk(lbm_handle *h, const char *path);

/* OutputCSV (lbm.cpp:3169-3186): "time,error" rows, time = (i+1) time_step. */
lbm_status lbmgpu_output_csv(const char *path, const double *values, int n, double time_step);
/* Rigid body: {xc[3], v[3], omega[3]}. */
lbm_status lbmgpu_get_body(lbm_handle *h, double out[9]);
/* Marker positions [3][n]. */
lbm_status lbmgpu_get_markers(lbm_handle *h, double *xyz);

lbm_status lbmgpu_status(lbm_handle *h, uint32_t *flags);
lbm_status lbmgpu_sync(lbm_handle *h);
lbm_status lbmgpu_steps_done(lbm_handle *h, long long *steps);
lbm_status lbmgpu_device_bytes(lbm_handle *h, size_t *bytes);
/* x-cells per thread the fused step uses on this handle (lbm_config.cells_per_thread after the
 * lattice and storage checks; 1 = one cell per thread).  No counterpart in the reference. */
lbm_status lbmgpu_cells_per_thread(lbm_handle *h, int *cells);

/* Page-locked host buffers for fast host<->device copies. */
lbm_status lbmgpu_host_alloc(size_t bytes, void **ptr);
lbm_status lbmgpu_host_free(void *ptr);

/* ------------------------------------------------------------------------
 * Batched cavities: many independent lid-driven cavities of uneven sizes
 * (each the reference's box with TYPE_S ghost walls and the lid on the
 * j = Ny+1 plane, lbm.cpp:1548-1551), advanced together by one persistent
 * launch per time step over a flattened tile queue, replayed through CUDA
 * graphs.  No counterpart in the reference (it runs one case per build);
 * each cavity follows LBM::Collision/Streaming/MacroProp.
 * ------------------------------------------------------------------------ */
typedef struct lbm_batch lbm_batch;
/* dims: [n][3] interior extents; tau: [n]; lid_u: lid velocity along x. */
lbm_status lbmgpu_batch_create(int n, const int *dims, const double *tau, double lid_u, int storage,
                               lbm_batch **out);
lbm_status lbmgpu_batch_destroy(lbm_batch *b);
lbm_status lbmgpu_batch_init(lbm_batch *b);
lbm_status lbmgpu_batch_step(lbm_batch *b, int nsteps);
lbm_status lbmgpu_batch_step_timed(lbm_batch *b, int nsteps, double *ms);
/* Choose threads per tile and grid shape by timing; chosen = {threads, grid}.
 * Advances the state: re-initialise afterwards. */
lbm_status lbmgpu_batch_autotune(lbm_batch *b, int *chosen);
/* rho, ux, uy, uz of one cavity ([4][cells], x fastest). */
lbm_status lbmgpu_batch_download(lbm_batch *b, int problem, float *host);
/* Per-cavity status words (LBM_STATUS_*). */
lbm_status lbmgpu_batch_status(lbm_batch *b, uint32_t *flags);
lbm_status lbmgpu_batch_info(lbm_batch *b, long long *total_cells, long long *steps);

/* Batched cavities without any device allocation (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- a host that gives
 * the solver buffers from its own pre-sized device pool and must stay inside
 * that pool's budget, or code that must not add the device-wide
 * synchronisation an allocation can cause while other work is in flight.
 * The caller owns the population buffers pop_a/pop_b (device memory, storage
 * type of `storage`): cavity p's populations start at element
 * base_p = 19 * sum_{q<p} S_q with S_q = 64 * ceil(Nx_q Ny_q Nz_q / 64), link l
 * of cell c at base_p + l * S_p + c, values stored as f - w.  nsteps steps run
 * A -> B -> A ...; the newest state ends in pop_a when nsteps is even, else in
 * pop_b.  first_step = 1 takes pop_a as the initial (pre-collision) state.
 * The library's working data (parameter table, tile table, status words) is
 * a fixed 8.4 MB device array that every GPU loading the library holds until
 * exit: at most 1024 cavities and 2^20 tiles of 256 cells; larger batches are
 * rejected with LBM_ERR_INVALID.  Every call clears the status words itself
 * and rewrites the tables, so nothing in that array has to start at zero.
 * Each call copies its tables from host memory, so it cannot be captured
 * into a CUDA graph: called on a stream that is being captured it returns
 * LBM_ERR_STATE and enqueues nothing.  All calls share
 * the array: calls that overlap on the GPU race.  status_out (host, n words,
 * may be NULL) receives the per-cavity status words; stream may be NULL (the
 * default stream).  Allocates nothing. */
lbm_status lbmgpu_batch_step_noalloc(int n, const int *dims, const double *tau, double lid_u, int storage,
                                     void *pop_a, void *pop_b, int first_step, int nsteps, uint32_t *status_out,
                                     void *stream);

/* ------------------------------------------------------------------------
 * Serving loop: requests (lid-driven cavities or channels with a fixed
 * sphere) arrive on a wall-clock schedule; each is admitted as soon as it has
 * arrived, a slot is free and its device memory fits the budget, keeps its
 * state on the device and is advanced in chunks on its own stream while the
 * others run (continuous batching).  No counterpart in the reference.
 * ------------------------------------------------------------------------ */
enum { LBM_SERVE_CAVITY = 0, LBM_SERVE_SPHERE = 1 };

typedef struct lbm_serve_request {
    double arrival_s;  /* arrival time, seconds after the start of the run; sorted */
    int kind;          /* LBM_SERVE_CAVITY or LBM_SERVE_SPHERE */
    int nx, ny, nz;
    double reynolds;   /* cavity: lid 0.05 and nx; sphere: inflow 0.05 and D = floor(ny / 6.4) */
    int steps;
    int storage;       /* LBM_STORE_* */
    float *fields;     /* optional: rho, ux, uy, uz of the result, [4][cells] */
} lbm_serve_request;

typedef struct lbm_serve_options {
    double hbm_budget_bytes; /* admission budget (0: unlimited) */
    int max_active;          /* solves in flight at once */
    int chunk_steps;         /* steps issued per solve per pass */
    double time_limit_s;     /* stop admitting and issuing after this (0: none) */
    int sphere_markers;      /* markers per sphere (0: about pi D^2) */
    int m_max;               /* IBM iterations for spheres (0: 3) */
} lbm_serve_options;

typedef struct lbm_serve_result {
    double admit_s, finish_s; /* -1 when it never happened */
    int status;               /* lbm_status of the request (LBM_ERR_STATE: cut by the time limit) */
    uint32_t flags;           /* device status word at the end */
    double drag;              /* sphere: x force of the last step (sum of -F_m ds) */
} lbm_serve_result;

/* Run the whole request trace; lattice_updates = cells x steps issued. */
lbm_status lbmgpu_serve_run(const lbm_serve_request *reqs, int n, const lbm_serve_options *opt,
                            lbm_serve_result *out, double *lattice_updates);

/* The reference's ENERGY model on D3Q19 (#define ENERGY without D2Q9; its
 * Rayleigh_Benard case, LBM.h:222-242, lbm.cpp:1585-1643), a solver object
 * of its own.  It is built from the reference's ghost-inclusive cell arrays,
 * (nx+2)(ny+2)(nz+2) cells, x fastest, indexed like LBM::fluid[i][j][k], and
 * keeps the reference's periodic modulo over that whole grid.  f and g are
 * FP32.  Walls: a TYPE_S cell whose type_Energy is TYPE_T is a Dirichlet
 * wall (lbm.cpp:277-280) at Determine_Wall_Temperature's T (lbm.cpp:965-981);
 * TYPE_Q a Neumann wall with j.n = 0 (lbm.cpp:281-288, 983-1028), evaluated
 * in the reference's serial push order; any other type an adiabatic wall
 * (its links keep their initial values).  With g_beta != 0, MacroProp sets
 * F_y = g_beta (T - T_star) on every cell, walls included (lbm.cpp:803-805),
 * so walls report u = F / (2 rho) and bounce back as moving walls from the
 * third streaming on. */
typedef struct lbm_energy3d lbm_energy3d;
typedef struct lbm_energy3d_setup {
    int nx, ny, nz;             /* interior cells */
    double tau, tau_g, cp;      /* tau; LBM.h's tau_g = 0.5 + alpha / cs2 and cp = k / (rho0 alpha) */
    double g_beta, T_star;      /* MacroProp's buoyancy; g_beta = 0: the set-up force stays */
    const uint8_t *type;        /* TYPE_F (0) or TYPE_S (1) */
    const uint8_t *type_energy; /* of TYPE_S cells: TYPE_T (6), TYPE_Q (7), other */
    const double *T;            /* set-up temperature, walls included */
    const double *rho;          /* set-up density; NULL: 1 */
    const double *u;            /* set-up velocity [3][cells]; NULL: 0 */
    const double *F;            /* set-up force [3][cells]; NULL: 0 */
    int graph_steps;            /* steps per captured CUDA graph from the third step on (rounded up to
                                   even, at most 1000); 0 = 10, <0 = every step launched on its own */
} lbm_energy3d_setup;
/* Creates the solver and runs LBM::Init on the set-up.  LBM_ERR_UNSUPPORTED
 * for other cell types, or a wall cell next to fluid without a solid
 * neighbour (its Determine_Wall_Temperature would divide by zero). */
lbm_status lbmgpu_energy3d_create(const lbm_energy3d_setup *setup, lbm_energy3d **out);
lbm_status lbmgpu_energy3d_init(lbm_energy3d *e);
/* nsteps of Collision, Streaming, MacroProp (main.cpp:213-220). */
lbm_status lbmgpu_energy3d_step(lbm_energy3d *e, int nsteps);
lbm_status lbmgpu_energy3d_step_timed(lbm_energy3d *e, int nsteps, double *ms);
/* LBM_FIELD_RHO .. LBM_FIELD_QZ after the last streaming and MacroProp, on
 * the whole ghost-inclusive grid, walls included: MacroProp's values on a
 * wall (lbm.cpp:657-806) are the sums of its initial populations, with
 * u = u_set + F / (2 rho) and q = 0. */
lbm_status lbmgpu_energy3d_download(lbm_energy3d *e, int field, double *host);
lbm_status lbmgpu_energy3d_status(lbm_energy3d *e, uint32_t *flags);
lbm_status lbmgpu_energy3d_destroy(lbm_energy3d *e);

const char *lbmgpu_last_error(void);
/* 2: lbm_config.cells_per_thread and lbm_ibm_config.virtual_mass appended
 * 3: lbm_energy3d (the ENERGY model on D3Q19) added */
int lbmgpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* LBMGPU_H */
