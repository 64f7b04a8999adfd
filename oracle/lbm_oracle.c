/*
 * lbm_oracle.c -- FP64 CPU restatement of the reference LBM time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle: the CUDA
 * product path never links, loads or calls it.  Only tests/, the smoke check
 * in __graft_entry__.py and the cpu_baseline leg of bench.py use it, and only
 * as the reference results are compared with (or as the timed CPU baseline).
 *
 * It restates, in plain C over flat arrays, the algorithm of the reference
 * solver (DestinyFlow01/Lattice-Boltzmann-Method---Graduate-FSI-):
 *   - LBM::Init                       lbm.cpp:31-57
 *   - LBM::Collision / ConvLBM        lbm.cpp:60-119  (BGK + Guo forcing)
 *   - LBM::Calc_feq (third order)     lbm.cpp:628-633
 *   - LBM::Streaming (push, halfway bounce-back with moving wall)
 *                                     lbm.cpp:182-296
 *   - LBM::Determine_Wall_Velocity    lbm.cpp:941-962
 *   - LBM::MacroProp                  lbm.cpp:657-679
 *   - kernel (4-point Peskin delta)   lbm.cpp:1095-1102
 *   - NearestLatticeCoordinate        lbm.cpp:1074-1092
 *   - Calc_AverageDensity             lbm.cpp:1105-1132
 *   - IBLBM implicit multi-direct forcing + added mass + Cl/Cd
 *                                     lbm.cpp:1135-1167, 1259-1416
 * with the same cell types, lattice ordering and operation order, so that on
 * cases the reference can express (3D cavity, 2D IBM cylinder) it agrees with
 * the reference build to rounding.
 *
 * New physics that the reference does not have (3D IBM sphere, D3Q7 thermal
 * population with Boussinesq force, thermal IBM, FP64 Newton-Euler rigid body,
 * true zero-gradient outlet) is restated here from the literature and defines
 * the semantics that the GPU path must reproduce:
 *   - D3Q7 advection-diffusion BGK, c_s^2 = 1/4 (w0 = 1/4, w1..6 = 1/8),
 *     tau_g = 0.5 + alpha / c_s^2, source term with the (1 - 1/(2 tau_g))
 *     factor (Seta 2013 style), T = sum g + Q/2.
 *   - Boussinesq body force F = g_beta * (T - T0) along the gravity axis,
 *     the form of lbm.cpp:804-805.
 *   - Rigid-body update with the internal-fluid treatment of Kempe &
 *     Froehlich (J. Comput. Phys. 231, 2012):
 *       rho_s V_s dV/dt = F_h + d/dt(int u dV) + (rho_s - rho_f) V_s g
 *       I_p dOmega/dt   = T_h + d/dt(int r x u dV).
 *   - Fibonacci (golden-angle) sphere markers with area weight pi D^2 / N.
 *
 * Compile with -ffp-contract=off so that x86 and aarch64 give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Cell types: LBM.h:505-515 (TYPE_F .. TYPE_Q).  ORC_OUTZG is new: a ghost
 * cell that repeats the post-collision populations of the interior cell next
 * to it (zero-gradient outlet). */
enum { ORC_F = 0, ORC_S = 1, ORC_OUT = 2, ORC_IN = 3, ORC_P = 4, ORC_L = 5, ORC_T = 6, ORC_Q = 7, ORC_OUTZG = 8 };

/* D2Q9 and D3Q19 tables in the reference order: LBM.h:528-555. */
static const int CX9[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int CY9[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const int CZ9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
static const double W9[9] = {4.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9,
                             1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
static const int OPP9[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

static const int CX19[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0};
static const int CY19[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1};
static const int CZ19[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1};
static const double W19[19] = {1.0 / 3,  1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18, 1.0 / 18,
                               1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36,
                               1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};
static const int OPP19[19] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};

/* D3Q7 thermal lattice (new): rest + 6 axis links, in the order of the first
 * seven D3Q19 links. */
static const int CX7[7] = {0, 1, -1, 0, 0, 0, 0};
static const int CY7[7] = {0, 0, 0, 1, -1, 0, 0};
static const int CZ7[7] = {0, 0, 0, 0, 0, 1, -1};
static const double W7[7] = {0.25, 0.125, 0.125, 0.125, 0.125, 0.125, 0.125};
static const int OPP7[7] = {0, 2, 1, 4, 3, 6, 5};
#define CS2T 0.25

/* PI as truncated in the reference (LBM.h:74). */
#define REF_PI 3.14159265

typedef struct orc {
    int q;               /* 9 or 19 */
    const int *cx, *cy, *cz, *opp;
    const double *w;
    int nx, ny, nz;      /* interior extent */
    int NX, NY, NZ;      /* with one ghost layer per face */
    long ncell;
    double tau;
    double cs2, cs2_3;   /* cs2 = dx^2/(3 dt^2) (LBM.h:86) and pow(cs2,3) */
    uint8_t *type;
    double *rho, *ux, *uy, *uz, *Fx, *Fy, *Fz;
    double *f, *fs;      /* [q][ncell] */
    double body[3];      /* uniform body force added in MacroProp (Poiseuille-like) */
    /* thermal (D3Q7) */
    int thermal;
    double tau_g, T0, gbeta[3];
    double *T, *Qh, *g, *gs;
    /* the reference's own thermal model (ENERGY): temperature populations on
     * the flow lattice, viscous heating, Dirichlet walls */
    int energy, ebuoy;
    int force_all;             /* Poiseuille_Flow: the body force is set on every cell */
    double etau_g, ecp, enu;
    double eg_beta, eT_star;   /* Rayleigh_Benard buoyancy F_y = g beta (T - T*) */
    double *eg, *egs, *fvis;   /* [q][ncell] */
    double *hq;                /* [3][ncell] heat flux sum g c */
    uint8_t *type_e;           /* type_Energy: ORC_T (Dirichlet) or ORC_Q (Neumann) on walls */
    double ejdn;               /* the Neumann walls' j . n (LBM.h's j_dot_n) */
} orc;

static inline long IDX(const orc *o, int i, int j, int k) {
    return (long)i + (long)o->NX * ((long)j + (long)o->NY * (long)k);
}

orc *orc_create(int q, int nx, int ny, int nz, double tau) {
    orc *o = (orc *)calloc(1, sizeof(orc));
    if (!o) return NULL;
    o->q = q;
    if (q == 9) {
        o->cx = CX9; o->cy = CY9; o->cz = CZ9; o->w = W9; o->opp = OPP9;
    } else {
        o->q = 19;
        o->cx = CX19; o->cy = CY19; o->cz = CZ19; o->w = W19; o->opp = OPP19;
    }
    o->nx = nx; o->ny = ny; o->nz = nz;
    o->NX = nx + 2; o->NY = ny + 2; o->NZ = nz + 2;
    o->ncell = (long)o->NX * o->NY * o->NZ;
    o->tau = tau;
    o->cs2 = pow(1.0, 2) / (3 * pow(1.0, 2));
    o->cs2_3 = pow(o->cs2, 3);
    long n = o->ncell;
    o->type = (uint8_t *)calloc(n, 1);
    o->rho = (double *)malloc(n * sizeof(double));
    o->ux = (double *)calloc(n, sizeof(double));
    o->uy = (double *)calloc(n, sizeof(double));
    o->uz = (double *)calloc(n, sizeof(double));
    o->Fx = (double *)calloc(n, sizeof(double));
    o->Fy = (double *)calloc(n, sizeof(double));
    o->Fz = (double *)calloc(n, sizeof(double));
    o->f = (double *)calloc((size_t)o->q * n, sizeof(double));
    o->fs = (double *)calloc((size_t)o->q * n, sizeof(double));
    for (long c = 0; c < n; c++) o->rho[c] = 1.0; /* LATTICE default density (LBM.h:561) */
    return o;
}

void orc_enable_thermal(orc *o, double tau_g, double T0, double gbx, double gby, double gbz) {
    long n = o->ncell;
    o->thermal = 1;
    o->tau_g = tau_g; o->T0 = T0;
    o->gbeta[0] = gbx; o->gbeta[1] = gby; o->gbeta[2] = gbz;
    o->T = (double *)calloc(n, sizeof(double));
    o->Qh = (double *)calloc(n, sizeof(double));
    o->g = (double *)calloc(7 * (size_t)n, sizeof(double));
    o->gs = (double *)calloc(7 * (size_t)n, sizeof(double));
}

/* The reference's ENERGY thermal model (LBM.h:58): g on the flow lattice.
 * T (fluid[..].T) must be set per cell by the caller, walls included. */
void orc_enable_energy(orc *o, double tau_g, double cp, double nu) {
    long n = o->ncell;
    o->energy = 1;
    o->etau_g = tau_g; o->ecp = cp; o->enu = nu;
    if (!o->T) o->T = (double *)calloc(n, sizeof(double));
    o->eg = (double *)calloc((size_t)o->q * n, sizeof(double));
    o->egs = (double *)calloc((size_t)o->q * n, sizeof(double));
    o->fvis = (double *)calloc((size_t)o->q * n, sizeof(double));
    o->hq = (double *)calloc(3 * (size_t)n, sizeof(double));
    o->type_e = (uint8_t *)calloc(n, 1);
}

void orc_free(orc *o) {
    if (!o) return;
    free(o->type); free(o->rho); free(o->ux); free(o->uy); free(o->uz);
    free(o->Fx); free(o->Fy); free(o->Fz); free(o->f); free(o->fs);
    free(o->T); free(o->Qh); free(o->g); free(o->gs);
    free(o->eg); free(o->egs); free(o->fvis); free(o->hq); free(o->type_e);
    free(o);
}

/* Poiseuille_Flow's force update on every cell (lbm.cpp:800-801). */
void orc_force_all(orc *o, int on) { o->force_all = on; }

/* Rayleigh_Benard's force update (lbm.cpp:803-805). */
void orc_energy_buoyancy(orc *o, double g_beta, double T_star) {
    o->ebuoy = 1;
    o->eg_beta = g_beta; o->eT_star = T_star;
}

/* Accessors for the ctypes wrapper. */
long orc_ncell(orc *o) { return o->ncell; }
uint8_t *orc_types(orc *o) { return o->type; }
uint8_t *orc_types_energy(orc *o) { return o->type_e; }
double *orc_field(orc *o, int which) {
    switch (which) {
    case 0: return o->rho;
    case 1: return o->ux;
    case 2: return o->uy;
    case 3: return o->uz;
    case 4: return o->Fx;
    case 5: return o->Fy;
    case 6: return o->Fz;
    case 7: return o->f;
    case 8: return o->fs;
    case 9: return o->T;
    case 10: return o->g;
    case 11: return o->gs;
    case 12: return o->Qh;
    case 13: return o->eg;
    case 14: return o->hq;
    case 15: return o->egs;
    case 16: return o->fvis;
    default: return NULL;
    }
}
void orc_set_body_force(orc *o, double fx, double fy, double fz) {
    o->body[0] = fx; o->body[1] = fy; o->body[2] = fz;
}

/* Third-order equilibrium, LBM::Calc_feq (lbm.cpp:628-633), same operation order. */
static inline double feq3(const orc *o, double rho, double ux, double uy, double uz, int l) {
    double cs2 = o->cs2;
    double u_dot_u = ux * ux + uy * uy + uz * uz;
    double c_dot_u = ux * o->cx[l] + uy * o->cy[l] + uz * o->cz[l];
    return rho * o->w[l] *
           (1 + c_dot_u / cs2 + (c_dot_u * c_dot_u) / (2 * cs2 * cs2) - u_dot_u / (2 * cs2) +
            pow(c_dot_u, 3) / (6 * o->cs2_3) - c_dot_u * u_dot_u / (2 * cs2 * cs2));
}

double orc_feq(orc *o, double rho, double ux, double uy, double uz, int l) {
    return feq3(o, rho, ux, uy, uz, l);
}

/* D3Q7 equilibrium (new): w_i T (1 + c.u / c_s^2). */
static inline double geq7(double T, double ux, double uy, double uz, int l) {
    return W7[l] * T * (1.0 + (CX7[l] * ux + CY7[l] * uy + CZ7[l] * uz) / CS2T);
}

/* LBM::Determine_Wall_Temperature, lbm.cpp:965-981: mean T of the solid
 * neighbours of a cell (periodic modulo over N+2). */
static double wall_temperature(const orc *o, int i, int j, int k) {
    int num = 0;
    double Tw = 0;
    for (int l = 0; l < o->q; l++) {
        int in = (i + o->cx[l] + o->NX) % o->NX;
        int jn = (j + o->cy[l] + o->NY) % o->NY;
        int kn = (k + o->cz[l] + o->NZ) % o->NZ;
        long nb = IDX(o, in, jn, kn);
        if (o->type[nb] == ORC_S) {
            Tw += o->T[nb];
            num++;
        }
    }
    Tw /= num;
    return Tw;
}

/* LBM::Calc_geq, lbm.cpp:636-653: rho w T (cubic equilibrium shape), with
 * the cell's T and u, or for a solid type the wall temperature of the cell
 * and the given wall velocity. */
static double energy_geq(const orc *o, int i, int j, int k, int l, int wall, const double uw[3]) {
    long c = IDX(o, i, j, k);
    double T, ux, uy, uz;
    if (wall) {
        T = wall_temperature(o, i, j, k);
        ux = uw[0]; uy = uw[1]; uz = uw[2];
    } else {
        T = o->T[c];
        ux = o->ux[c]; uy = o->uy[c]; uz = o->uz[c];
    }
    double cs2 = o->cs2;
    double u_dot_u = pow(ux, 2) + pow(uy, 2) + pow(uz, 2);
    double c_dot_u = ux * o->cx[l] + uy * o->cy[l] + uz * o->cz[l];
    return o->rho[c] * o->w[l] * T *
           (1 + c_dot_u / cs2 + pow(c_dot_u, 2) / (2 * cs2 * cs2) - u_dot_u / (2 * cs2) +
            pow(c_dot_u, 3) / (6 * o->cs2_3) - c_dot_u * u_dot_u / (2 * cs2 * cs2));
}

/* LBM::Init, lbm.cpp:31-57: f = f* = feq(rho,u) on every cell, ghosts included. */
void orc_init(orc *o) {
    long n = o->ncell;
#pragma omp parallel for
    for (long c = 0; c < n; c++) {
        for (int l = 0; l < o->q; l++) {
            double fe = feq3(o, o->rho[c], o->ux[c], o->uy[c], o->uz[c], l);
            o->f[l * n + c] = fe;
            o->fs[l * n + c] = fe;
        }
        if (o->thermal) {
            for (int l = 0; l < 7; l++) {
                double ge = geq7(o->T[c], o->ux[c], o->uy[c], o->uz[c], l);
                o->g[l * n + c] = ge;
                o->gs[l * n + c] = ge;
            }
        }
    }
    if (o->energy) {
        /* g = g* = Calc_geq(cell type), the wall velocity zero (lbm.cpp:44-49) */
        const double zero[3] = {0, 0, 0};
#pragma omp parallel for collapse(2)
        for (int k = 0; k < o->NZ; k++)
            for (int j = 0; j < o->NY; j++)
                for (int i = 0; i < o->NX; i++) {
                    long c = IDX(o, i, j, k);
                    for (int l = 0; l < o->q; l++) {
                        double ge = energy_geq(o, i, j, k, l, o->type[c] == ORC_S, zero);
                        o->eg[l * n + c] = ge;
                        o->egs[l * n + c] = ge;
                    }
                }
    }
}

/* LBM::Collision + ConvLBM, lbm.cpp:60-119: BGK with Guo forcing on TYPE_F
 * cells, using the stored density, velocity and force.  Returns the number
 * of cells where feq < 0 (the reference terminates there, lbm.cpp:114-117). */
long orc_collide(orc *o) {
    long n = o->ncell, bad = 0;
    double omega = 1.0 / o->tau; /* dt/tau */
    double cs2 = o->cs2;
#pragma omp parallel for reduction(+ : bad)
    for (long c = 0; c < n; c++) {
        if (o->type[c] != ORC_F) continue;
        double rho = o->rho[c], ux = o->ux[c], uy = o->uy[c], uz = o->uz[c];
        double Fx = o->Fx[c], Fy = o->Fy[c], Fz = o->Fz[c];
        double F_dot_u = Fx * ux + Fy * uy + Fz * uz;
        for (int l = 0; l < o->q; l++) {
            double c_dot_u = ux * o->cx[l] + uy * o->cy[l] + uz * o->cz[l];
            double f_eq = feq3(o, rho, ux, uy, uz, l);
            double F_dot_c = Fx * o->cx[l] + Fy * o->cy[l] + Fz * o->cz[l];
            double Source = (1 - omega * 0.5) * o->w[l] *
                            (F_dot_c / cs2 + (F_dot_c) * (c_dot_u) / (cs2 * cs2) - F_dot_u / cs2);
            o->fs[l * n + c] = o->f[l * n + c] * (1 - omega) + omega * f_eq + Source * 1.0;
            if (f_eq < 0) bad++;
        }
        if (o->energy) {
            /* ENERGY part of ConvLBM (lbm.cpp:121-177): viscous dissipation
             * Phi = 2 nu rho S:S with S from the non-equilibrium part of f,
             * the source F_vis and its time derivative against the previous
             * step's F_vis */
            double S[3][3];
            const int *cc[3] = {o->cx, o->cy, o->cz};
            for (int row = 0; row < 3; row++)
                for (int col = 0; col < 3; col++) {
                    S[row][col] = 0;
                    if (col < row) continue;
                    for (int l = 0; l < o->q; l++) {
                        double f_eq = feq3(o, rho, ux, uy, uz, l);
                        S[row][col] += cc[row][l] * cc[col][l] * (o->f[l * n + c] - f_eq);
                    }
                }
            S[1][0] = S[0][1]; S[2][0] = S[0][2]; S[2][1] = S[1][2];
            for (int row = 0; row < 3; row++)
                for (int col = 0; col < 3; col++) S[row][col] = -S[row][col] / (2 * rho * o->tau * cs2);
            double Phi = 0;
            for (int row = 0; row < 3; row++)
                for (int col = 0; col < 3; col++) Phi += S[row][col] * S[row][col];
            Phi = 2 * o->enu * rho * Phi;
            const double tg = o->etau_g;
            const int ci = (int)(c % o->NX), cj = (int)((c / o->NX) % o->NY), ck = (int)(c / ((long)o->NX * o->NY));
            const double zero[3] = {0, 0, 0};
            for (int l = 0; l < o->q; l++) {
                double c_dot_u = ux * o->cx[l] + uy * o->cy[l] + uz * o->cz[l];
                double F_before = o->fvis[l * n + c];
                double F = o->w[l] * Phi / o->ecp * (1 + c_dot_u * (tg - 0.5) / (cs2 * tg));
                o->fvis[l * n + c] = F;
                double dF_dt = (F - F_before) / 1.0;
                double g_eq = energy_geq(o, ci, cj, ck, l, 0, zero);
                double gl = o->eg[l * n + c];
                o->egs[l * n + c] = gl - (gl - g_eq) / tg + 1.0 * F + 0.5 * pow(1.0, 2) * dF_dt;
            }
        }
        if (o->thermal) {
            /* D3Q7 BGK with heat source Qh (new physics). */
            double T = o->T[c], tg = o->tau_g;
            for (int l = 0; l < 7; l++) {
                double ge = geq7(T, ux, uy, uz, l);
                double gl = o->g[l * n + c];
                o->gs[l * n + c] = gl - (gl - ge) / tg + (1.0 - 0.5 / tg) * W7[l] * o->Qh[c];
            }
        }
    }
    return bad;
}

/* LBM::Determine_Wall_Velocity, lbm.cpp:941-962: mean velocity of the moving
 * solid neighbours of a fluid cell (a solid counts as moving when any of its
 * velocity components is non-zero). */
static void wall_velocity(const orc *o, int i, int j, int k, double uw[3]) {
    int num = 0;
    uw[0] = uw[1] = uw[2] = 0.0;
    for (int l = 0; l < o->q; l++) {
        int in = (i + o->cx[l] + o->NX) % o->NX;
        int jn = (j + o->cy[l] + o->NY) % o->NY;
        int kn = (k + o->cz[l] + o->NZ) % o->NZ;
        long nb = IDX(o, in, jn, kn);
        if (o->type[nb] == ORC_S) {
            if (o->ux[nb] != 0 || o->uy[nb] != 0 || o->uz[nb] != 0) {
                uw[0] += o->ux[nb]; uw[1] += o->uy[nb]; uw[2] += o->uz[nb];
                num++;
            }
        }
    }
    if (num != 0) { uw[0] /= num; uw[1] /= num; uw[2] /= num; }
}

/* Zero-gradient source (new): the interior cell next to a ORC_OUTZG ghost,
 * obtained by clamping every ghost coordinate into [1, n]. */
static long zg_source(const orc *o, int i, int j, int k) {
    if (i < 1) i = 1; if (i > o->nx) i = o->nx;
    if (j < 1) j = 1; if (j > o->ny) j = o->ny;
    if (k < 1) k = 1; if (k > o->nz) k = o->nz;
    return IDX(o, i, j, k);
}

/* LBM::Streaming, fluid part (lbm.cpp:182-296): push f* of every TYPE_F cell
 * to its TYPE_F neighbours; halfway bounce-back with the cell's wall velocity
 * on TYPE_S links (lbm.cpp:267-274).  Populations arriving from TYPE_IN /
 * TYPE_OUT ghosts are never written, as in the reference.  The face-BC loops
 * of lbm.cpp:299-624 only touch ghost cells that no fluid cell reads, so they
 * are not restated.  Extension: populations arriving from a ORC_OUTZG ghost
 * take the post-collision value of the clamped interior cell. */
/* LBM::Determine_Twall_Neumann, lbm.cpp:983-1028, for cell (i, j, k) in
 * the middle of the push: the normal is the mean of the directions of the
 * links that face a wall (cdotn_pos, the opposites of the solid links, not
 * normalised); the links not facing a wall contribute the cell's current g
 * -- this sweep's value where the source was visited earlier, the previous
 * sweep's otherwise --, the facing ones the wall equilibrium at T = 1 (cubic
 * shape, the cell's rho and the wall velocity); T_w = (j.n - sum_notpos) /
 * sum_pos, also written into the wall cell opposite the normal. */
static double twall_neumann(orc *o, int i, int j, int k, long c, const double uw[3]) {
    long n = o->ncell;
    int pos[27], npos = 0, is_pos[27] = {0};
    for (int l = 0; l < o->q; l++) {
        int in = (i + o->cx[l] + o->NX) % o->NX;
        int jn = (j + o->cy[l] + o->NY) % o->NY;
        int kn = (k + o->cz[l] + o->NZ) % o->NZ;
        if (o->type[IDX(o, in, jn, kn)] == ORC_S) {
            pos[npos++] = o->opp[l];
            is_pos[o->opp[l]] = 1;
        }
    }
    double nrm[3] = {0, 0, 0};
    for (int p = 0; p < npos; p++) {
        nrm[0] += o->cx[pos[p]];
        nrm[1] += o->cy[pos[p]];
        nrm[2] += o->cz[pos[p]];
    }
    nrm[0] /= npos; nrm[1] /= npos; nrm[2] /= npos;
    double sum_notpos = 0;
    for (int l = 0; l < o->q; l++) {
        if (is_pos[l]) continue;
        sum_notpos += o->eg[l * n + c] * (o->cx[l] * nrm[0] + o->cy[l] * nrm[1] + o->cz[l] * nrm[2]);
    }
    double cs2 = o->cs2, uu = uw[0] * uw[0] + uw[1] * uw[1] + uw[2] * uw[2];
    double sum_pos = 0;
    for (int p = 0; p < npos; p++) {
        int l = pos[p];
        double uc = uw[0] * o->cx[l] + uw[1] * o->cy[l] + uw[2] * o->cz[l];
        double eq = o->w[l] * o->rho[c] *
                    (1 + uc / cs2 + pow(uc, 2) / (2 * cs2 * cs2) - uu / (2 * cs2) + pow(uc, 3) / (6 * pow(cs2, 3)) -
                     uc * uu / (2 * cs2 * cs2));
        sum_pos += eq * (o->cx[l] * nrm[0] + o->cy[l] * nrm[1] + o->cz[l] * nrm[2]);
    }
    double Tw = (o->ejdn - sum_notpos) / sum_pos;
    for (int l = 0; l < o->q; l++) {
        int m = o->opp[l];
        if (o->cx[m] == nrm[0] && o->cy[m] == nrm[1] && o->cz[m] == nrm[2]) {
            int in = (i + o->cx[l] + o->NX) % o->NX;
            int jn = (j + o->cy[l] + o->NY) % o->NY;
            int kn = (k + o->cz[l] + o->NZ) % o->NZ;
            o->T[IDX(o, in, jn, kn)] = Tw;
            break;
        }
    }
    return Tw;
}

/* Streaming of one fluid cell (the body of orc_stream's loops). */
static void stream_cell(orc *o, int i, int j, int k) {
    long n = o->ncell;
    double cs2 = o->cs2;
    long c = IDX(o, i, j, k);
    if (o->type[c] != ORC_F) return;
    int have_uw = 0;
    double uw[3] = {0, 0, 0};
    for (int l = 0; l < o->q; l++) {
        int in = (i + o->cx[l] + o->NX) % o->NX;
        int jn = (j + o->cy[l] + o->NY) % o->NY;
        int kn = (k + o->cz[l] + o->NZ) % o->NZ;
        long nb = IDX(o, in, jn, kn);
        uint8_t t = o->type[nb];
        if (t == ORC_F) {
            o->f[l * n + nb] = o->fs[l * n + c];
            if (o->energy) o->eg[l * n + nb] = o->egs[l * n + c];
        } else if (t == ORC_S) {
            if (!have_uw) { wall_velocity(o, i, j, k, uw); have_uw = 1; }
            double uwall_dot_c = uw[0] * o->cx[l] + uw[1] * o->cy[l] + uw[2] * o->cz[l];
            o->f[o->opp[l] * n + c] = o->fs[l * n + c] - 2 * o->w[l] * uwall_dot_c / cs2;
            /* Dirichlet wall (type_Energy TYPE_T): anti-bounce-back
             * against the wall equilibrium (lbm.cpp:277-280) */
            if (o->energy && o->type_e[nb] == ORC_T) {
                double g_eq = energy_geq(o, i, j, k, l, 1, uw);
                o->eg[o->opp[l] * n + c] = -o->egs[l * n + c] + 2 * g_eq;
            } else if (o->energy && o->type_e[nb] == ORC_Q) {
                /* Neumann wall (lbm.cpp:281-288): the wall's T from
                 * the heat flux, and the unknown g as the
                 * second-order equilibrium of T_w; a wall of any
                 * other type_Energy (adiabatic) writes nothing */
                double Tw = twall_neumann(o, i, j, k, c, uw);
                o->T[nb] = Tw;
                double uu = uw[0] * uw[0] + uw[1] * uw[1] + uw[2] * uw[2];
                o->eg[o->opp[l] * n + c] =
                    o->w[l] * o->rho[c] * Tw *
                    (1 + uwall_dot_c / cs2 + pow(uwall_dot_c, 2) / (2 * cs2 * cs2) - uu / (2 * cs2));
            }
        }
        /* Pull-side view of the zero-gradient ghost: the
         * population of this cell arriving from direction l's
         * opposite neighbour. */
        int m = o->opp[l];
        if (t == ORC_OUTZG) {
            /* neighbour nb = x + c_l = x - c_m is the source of population m */
            long src = zg_source(o, in, jn, kn);
            if (o->type[src] == ORC_F) o->f[m * n + c] = o->fs[m * n + src];
        }
    }
    if (o->thermal) {
        for (int l = 0; l < 7; l++) {
            int in = (i + CX7[l] + o->NX) % o->NX;
            int jn = (j + CY7[l] + o->NY) % o->NY;
            int kn = (k + CZ7[l] + o->NZ) % o->NZ;
            long nb = IDX(o, in, jn, kn);
            uint8_t t = o->type[nb];
            if (t == ORC_F) {
                o->g[l * n + nb] = o->gs[l * n + c];
            } else if (t == ORC_S) {
                /* adiabatic wall: plain bounce-back of g */
                o->g[OPP7[l] * n + c] = o->gs[l * n + c];
            } else if (t == ORC_OUTZG) {
                int m = OPP7[l];
                long src = zg_source(o, in, jn, kn);
                if (o->type[src] == ORC_F) o->g[m * n + c] = o->gs[m * n + src];
            }
        }
    }
}

/* LBM::Streaming, fluid part.  With a Neumann wall the result depends on the
 * order the cells are visited in (twall_neumann reads this sweep's pushes),
 * so the loop runs in the reference's order, i outer, k inner, on one
 * thread; otherwise every write has one source and the loop runs in
 * parallel. */
void orc_stream(orc *o) {
    int neumann = 0;
    if (o->energy)
        for (long c = 0; c < o->ncell && !neumann; c++) neumann = o->type_e[c] == ORC_Q;
    if (neumann) {
        for (int i = 0; i < o->NX; i++)
            for (int j = 0; j < o->NY; j++)
                for (int k = 0; k < o->NZ; k++) stream_cell(o, i, j, k);
        return;
    }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < o->NZ; k++)
        for (int j = 0; j < o->NY; j++)
            for (int i = 0; i < o->NX; i++) stream_cell(o, i, j, k);
}

/* LBM::MacroProp, lbm.cpp:657-679: rho = sum f, u = (sum f c + F/2) / rho on
 * every cell.  With the thermal population (new physics): T = sum g, and the
 * force is refreshed before u, F = body + g_beta (T - T0) (consistent
 * Boussinesq coupling, cf. lbm.cpp:804-805).  Returns the number of cells with
 * rho outside [0, 100] (lbm.cpp:772-775). */
long orc_macro(orc *o) {
    long n = o->ncell, bad = 0;
#pragma omp parallel for reduction(+ : bad)
    for (long c = 0; c < n; c++) {
        double rho = 0, rho_ux = 0, rho_uy = 0, rho_uz = 0;
        for (int l = 0; l < o->q; l++) {
            double fl = o->f[l * n + c];
            rho += fl;
            rho_ux += fl * o->cx[l];
            rho_uy += fl * o->cy[l];
            rho_uz += fl * o->cz[l];
        }
        if (o->thermal) {
            double T = 0;
            for (int l = 0; l < 7; l++) T += o->g[l * n + c];
            o->T[c] = T;
            o->Qh[c] = 0.0;
            if (o->type[c] == ORC_F) {
                o->Fx[c] = o->body[0] + o->gbeta[0] * (T - o->T0);
                o->Fy[c] = o->body[1] + o->gbeta[1] * (T - o->T0);
                o->Fz[c] = o->body[2] + o->gbeta[2] * (T - o->T0);
            }
        } else if (o->type[c] == ORC_F && (o->body[0] != 0 || o->body[1] != 0 || o->body[2] != 0)) {
            o->Fx[c] = o->body[0]; o->Fy[c] = o->body[1]; o->Fz[c] = o->body[2];
        }
        if (o->energy) {
            /* T = sum g, q = sum g c on every cell (lbm.cpp:776-792) */
            double T = 0, gx = 0, gy = 0, gz = 0;
            for (int l = 0; l < o->q; l++) {
                double gl = o->eg[l * n + c];
                T += gl; gx += gl * o->cx[l]; gy += gl * o->cy[l]; gz += gl * o->cz[l];
            }
            o->T[c] = T;
            o->hq[c] = gx; o->hq[n + c] = gy; o->hq[2 * n + c] = gz;
        }
        o->rho[c] = rho;
        o->ux[c] = (rho_ux + 0.5 * 1.0 * o->Fx[c]) / rho;
        o->uy[c] = (rho_uy + 0.5 * 1.0 * o->Fy[c]) / rho;
        o->uz[c] = (rho_uz + 0.5 * 1.0 * o->Fz[c]) / rho;
        /* Poiseuille_Flow: F = -dp/dx on every cell, walls included, after u
         * took the previous force (lbm.cpp:800-801); a wall then reports
         * u = F / 2 rho from the second MacroProp on */
        if (o->force_all) {
            o->Fx[c] = o->body[0]; o->Fy[c] = o->body[1]; o->Fz[c] = o->body[2];
        }
        /* Rayleigh_Benard: F_y = g beta (T - T*) on every cell, after u took
         * the previous force (lbm.cpp:803-805) */
        if (o->energy && o->ebuoy) o->Fy[c] = o->eg_beta * (o->T[c] - o->eT_star);
        if (rho < 0 || rho > 100) bad++;
        if (o->energy && (o->T[c] < 0 || o->T[c] > 100)) bad++;
    }
    return bad;
}

/* One non-IBM time step in the reference order (main.cpp:214-220):
 * Collision -> Streaming -> MacroProp. */
long orc_step_plain(orc *o, int nsteps) {
    long bad = 0;
    for (int s = 0; s < nsteps; s++) {
        bad += orc_collide(o);
        orc_stream(o);
        bad += orc_macro(o);
    }
    return bad;
}

/* MEA_CD / MEA_CL, lbm.cpp:3085-3163 (momentum exchange on staircase solid
 * cells): over the fluid cells of the box [xmin,xmax] x [ymin,ymax] x
 * [zmin,zmax] (ghost-inclusive reference indices), every link l whose cell
 * i - c_l is TYPE_S adds (f*_l + f_opp(l)) c_l.  out = (sum x, sum y, sum z);
 * the reference's drag is -out[0] and its lift +out[1] (times dx^3/dt, then
 * divided by 1/2 rho0 u^2 times the area). */
void orc_mea(const orc *o, int xmin, int xmax, int ymin, int ymax, int zmin, int zmax, double out[3]) {
    long n = o->ncell;
    double sx = 0, sy = 0, sz = 0;
    for (int i = xmin; i <= xmax; ++i)
        for (int j = ymin; j <= ymax; ++j)
            for (int k = zmin; k <= zmax; ++k) {
                long c = IDX(o, i, j, k);
                if (o->type[c] != ORC_F) continue;
                for (int l = 0; l < o->q; ++l) {
                    long nb = IDX(o, i - o->cx[l], j - o->cy[l], k - o->cz[l]);
                    if (o->type[nb] != ORC_S) continue;
                    const double t = o->fs[l * n + c] + o->f[o->opp[l] * n + c];
                    sx += t * o->cx[l];
                    sy += t * o->cy[l];
                    sz += t * o->cz[l];
                }
            }
    out[0] = sx;
    out[1] = sy;
    out[2] = sz;
}

/* ------------------------------------------------------------------------ */
/* Immersed boundary                                                         */
/* ------------------------------------------------------------------------ */

/* kernel(r), lbm.cpp:1095-1102: 4-point Peskin delta. */
double orc_kernel(double r) {
    double d, a = fabs(r);
    if (a >= 0 && a <= 1) d = (3 - 2 * a + sqrt(1 + 4 * a - 4 * r * r)) / 8;
    else if (a >= 1 && a <= 2) d = (5 - 2 * a - sqrt(-7 + 12 * a - 4 * r * r)) / 8;
    else d = 0;
    return d;
}

typedef struct orc_markers {
    int n;
    double *x, *y, *z;          /* positions */
    double *nx, *ny, *nz;       /* outward normals */
    double *ds;                 /* area (3D) or arc length (2D) weight */
    double *udx, *udy, *udz;    /* desired velocity u_boundary_des */
    double *ubx, *uby, *ubz;    /* interpolated velocity u_boundary */
    double *Fbx, *Fby, *Fbz;    /* marker force F_boundary */
    double *Td, *Tb, *Qb;       /* thermal: desired T, interpolated T, heat source */
} orc_markers;

/* IBM options.  box_* bound the Eulerian nodes that take part (the reference
 * uses [center -/+ D], lbm.cpp:1165-1167).  lit_sign = 1 reproduces the sign
 * convention of lbm.cpp:1347-1352 (force -Fm, velocity +Fm/2rho); 0 uses the
 * consistent +Fm for both.  rho_mode = 1 takes the density at
 * NearestLatticeCoordinate over the whole box (lbm.cpp:1315-1317); 0 takes
 * the delta-interpolated density at the marker. */
typedef struct orc_ibm_opts {
    int box_lo[3], box_hi[3];
    int m_max;
    int lit_sign;
    int rho_mode;
    int thermal;       /* also force the temperature towards Td */
    int use_avg_density; /* 1: Calc_AverageDensity for the added-mass term */
    double vsolid;     /* V_solid for the added-mass term */
    double vcm_new[3], vcm_old[3];
    int scheme;        /* 0: implicit multi-direct forcing; 1: explicit direct forcing */
} orc_ibm_opts;

static inline int ibm_node_ok(uint8_t t) { return t == ORC_F || t == ORC_IN || t == ORC_OUT || t == ORC_OUTZG; }

/* Interpolate a field sum over the stencil |r| < 2 of marker m, restricted to
 * the box and to F/IN/OUT nodes, summed in x-outer, z-inner order as the
 * reference's box loop (lbm.cpp:1288-1309). */
static void interp3(const orc *o, const orc_ibm_opts *op, double X, double Y, double Z,
                    const double *a, const double *b, const double *c3, double out[3]) {
    double s0 = 0, s1 = 0, s2 = 0;
    if (!(X > -2 && X < o->NX + 2 && Y > -2 && Y < o->NY + 2 && Z > -2 && Z < o->NZ + 2)) {
        out[0] = out[1] = out[2] = NAN; /* marker left the lattice */
        return;
    }
    int i0 = (int)floor(X) - 1, j0 = (int)floor(Y) - 1, k0 = (int)floor(Z) - 1;
    for (int i = i0; i <= i0 + 3; i++) {
        if (i < op->box_lo[0] || i > op->box_hi[0]) continue;
        double kx = orc_kernel((i * 1.0 - X) / 1.0);
        for (int j = j0; j <= j0 + 3; j++) {
            if (j < op->box_lo[1] || j > op->box_hi[1]) continue;
            double ky = orc_kernel((j * 1.0 - Y) / 1.0);
            for (int k = k0; k <= k0 + 3; k++) {
                if (k < op->box_lo[2] || k > op->box_hi[2]) continue;
                long cidx = IDX(o, i, j, k);
                if (!ibm_node_ok(o->type[cidx])) continue;
                double kz = orc_kernel((k * 1.0 - Z) / 1.0);
                s0 += a[cidx] * kx * ky * kz;
                if (b) s1 += b[cidx] * kx * ky * kz;
                if (c3) s2 += c3[cidx] * kx * ky * kz;
            }
        }
    }
    out[0] = s0; out[1] = s1; out[2] = s2;
}

/* NearestLatticeCoordinate, lbm.cpp:1074-1092: the box node farthest along
 * the marker normal (dot >= best and dot > 0; later nodes win ties). */
static long nearest_node(const orc *o, const orc_ibm_opts *op, const orc_markers *mk, int m) {
    double dot = 0;
    int bi = 0, bj = 0, bk = 1;
    for (int x = op->box_lo[0]; x <= op->box_hi[0]; x++)
        for (int y = op->box_lo[1]; y <= op->box_hi[1]; y++)
            for (int z = op->box_lo[2]; z <= op->box_hi[2]; z++) {
                double vx = x - mk->x[m], vy = y - mk->y[m], vz = z - mk->z[m];
                double d = vx * mk->nx[m] + vy * mk->ny[m] + vz * mk->nz[m];
                if (d >= dot && d > 0) { bi = x; bj = y; bk = z; dot = d; }
            }
    return IDX(o, bi, bj, bk);
}

/* Calc_AverageDensity, lbm.cpp:1105-1132: mean density over box nodes on the
 * inner side of every marker. */
static double average_density(const orc *o, const orc_ibm_opts *op, const orc_markers *mk) {
    double rho = 0;
    long number = 0;
    for (int i = op->box_lo[0]; i <= op->box_hi[0]; i++)
        for (int j = op->box_lo[1]; j <= op->box_hi[1]; j++)
            for (int k = op->box_lo[2]; k <= op->box_hi[2]; k++) {
                int neg = 1;
                for (int m = 0; m < mk->n; m++) {
                    double d = (i - mk->x[m]) * mk->nx[m] + (j - mk->y[m]) * mk->ny[m] + (k - mk->z[m]) * mk->nz[m];
                    if (d > 0) { neg = 0; break; }
                }
                if (neg) { rho += o->rho[IDX(o, i, j, k)]; number++; }
            }
    return rho / number;
}

/* IBLBM implicit multi-direct forcing (lbm.cpp:1259-1398), restated for a 3D
 * stencil.  Writes the unforced moments, spreads the marker forces and leaves
 * rho, u (force-corrected) and F on the lattice for the following collision.
 * force_out[0..2] = sum over iterations of -F_m ds_m dx (the reference's
 * Drag/Lift accumulators, plus the added-mass term), force_out[3..5] = the
 * torque of the same forces about (cx, cy, cz) (for the rigid body),
 * force_out[6] = total heat released by the thermal markers. */
void orc_ibm_step(orc *o, orc_markers *mk, const orc_ibm_opts *op, const double center[3], double force_out[7]) {
    long n = o->ncell;
    double drag[3] = {0, 0, 0}, torque[3] = {0, 0, 0}, heat = 0;
    /* (i) unforced moments on F/IN/OUT cells, F reset (lbm.cpp:1262-1285).
     * With the thermal population the Boussinesq force stays in F and in u. */
#pragma omp parallel for
    for (long c = 0; c < n; c++) {
        if (!ibm_node_ok(o->type[c])) continue;
        double rho = 0, r0 = 0, r1 = 0, r2 = 0;
        for (int l = 0; l < o->q; l++) {
            double fl = o->f[l * n + c];
            rho += fl; r0 += fl * o->cx[l]; r1 += fl * o->cy[l]; r2 += fl * o->cz[l];
        }
        double Fb[3] = {o->body[0], o->body[1], o->body[2]};
        if (o->thermal) {
            double T = 0;
            for (int l = 0; l < 7; l++) T += o->g[l * n + c];
            o->T[c] = T;
            o->Qh[c] = 0.0;
            Fb[0] += o->gbeta[0] * (T - o->T0);
            Fb[1] += o->gbeta[1] * (T - o->T0);
            Fb[2] += o->gbeta[2] * (T - o->T0);
        }
        o->rho[c] = rho;
        if (Fb[0] == 0 && Fb[1] == 0 && Fb[2] == 0) {
            o->ux[c] = r0 / rho; o->uy[c] = r1 / rho; o->uz[c] = r2 / rho;
        } else {
            o->ux[c] = (r0 + 0.5 * Fb[0]) / rho; o->uy[c] = (r1 + 0.5 * Fb[1]) / rho; o->uz[c] = (r2 + 0.5 * Fb[2]) / rho;
        }
        o->Fx[c] = Fb[0]; o->Fy[c] = Fb[1]; o->Fz[c] = Fb[2];
    }
    int N = mk->n;
    double *rho_m = (double *)malloc(N * sizeof(double));
    /* (ii) unforced interpolation (lbm.cpp:1288-1309) and marker densities */
#pragma omp parallel for
    for (int m = 0; m < N; m++) {
        double u3[3];
        interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->ux, o->uy, o->uz, u3);
        mk->ubx[m] = u3[0]; mk->uby[m] = u3[1]; mk->ubz[m] = u3[2];
        if (op->rho_mode == 1) {
            rho_m[m] = o->rho[nearest_node(o, op, mk, m)];
        } else {
            double r3[3];
            interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->rho, NULL, NULL, r3);
            rho_m[m] = r3[0];
        }
        if (op->thermal) {
            double t3[3];
            interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->T, NULL, NULL, t3);
            mk->Tb[m] = t3[0];
        }
    }
    /* lattice scratch for the spread increments (Fm, lbm.cpp:1333-1344) */
    int bx = op->box_hi[0] - op->box_lo[0] + 1, by = op->box_hi[1] - op->box_lo[1] + 1,
        bz = op->box_hi[2] - op->box_lo[2] + 1;
    if (bx < 1 || by < 1 || bz < 1) bx = by = bz = 1; /* body outside the lattice: nothing to spread */
    long nb = (long)bx * by * bz;
    double *Fm = (double *)calloc(4 * nb, sizeof(double));
    double sgn = op->lit_sign ? -1.0 : 1.0;
    for (int it = 1; it <= op->m_max; it++) {
        /* boundary force (lbm.cpp:1314-1324) */
        for (int m = 0; m < N; m++) {
            double rho = rho_m[m];
            mk->Fbx[m] = 2 * rho * (mk->udx[m] - mk->ubx[m]) / 1.0;
            mk->Fby[m] = 2 * rho * (mk->udy[m] - mk->uby[m]) / 1.0;
            mk->Fbz[m] = 2 * rho * (mk->udz[m] - mk->ubz[m]) / 1.0;
            double dv = 1.0 * mk->ds[m];
            double fx = -mk->Fbx[m] * dv, fy = -mk->Fby[m] * dv, fz = -mk->Fbz[m] * dv;
            drag[0] += fx; drag[1] += fy; drag[2] += fz;
            double rx = mk->x[m] - center[0], ry = mk->y[m] - center[1], rz = mk->z[m] - center[2];
            torque[0] += ry * fz - rz * fy;
            torque[1] += rz * fx - rx * fz;
            torque[2] += rx * fy - ry * fx;
            if (op->thermal) {
                mk->Qb[m] = 2 * (mk->Td[m] - mk->Tb[m]) / 1.0;
                heat += mk->Qb[m] * dv;
            }
        }
        /* spreading (lbm.cpp:1331-1360): marker order ascending per node */
        memset(Fm, 0, 4 * nb * sizeof(double));
        for (int m = 0; m < N; m++) {
            double X = mk->x[m], Y = mk->y[m], Z = mk->z[m];
            if (!(X > -2 && X < o->NX + 2 && Y > -2 && Y < o->NY + 2 && Z > -2 && Z < o->NZ + 2)) continue;
            int i0 = (int)floor(X) - 1, j0 = (int)floor(Y) - 1, k0 = (int)floor(Z) - 1;
            for (int i = i0; i <= i0 + 3; i++) {
                if (i < op->box_lo[0] || i > op->box_hi[0]) continue;
                double kx = orc_kernel(i - X);
                for (int j = j0; j <= j0 + 3; j++) {
                    if (j < op->box_lo[1] || j > op->box_hi[1]) continue;
                    double ky = orc_kernel(j - Y);
                    for (int k = k0; k <= k0 + 3; k++) {
                        if (k < op->box_lo[2] || k > op->box_hi[2]) continue;
                        if (!ibm_node_ok(o->type[IDX(o, i, j, k)])) continue;
                        double kz = orc_kernel(k - Z);
                        long b = (i - op->box_lo[0]) + (long)bx * ((j - op->box_lo[1]) + (long)by * (k - op->box_lo[2]));
                        Fm[4 * b + 0] += mk->Fbx[m] * mk->ds[m] * kx * ky * kz;
                        Fm[4 * b + 1] += mk->Fby[m] * mk->ds[m] * kx * ky * kz;
                        Fm[4 * b + 2] += mk->Fbz[m] * mk->ds[m] * kx * ky * kz;
                        if (op->thermal) Fm[4 * b + 3] += mk->Qb[m] * mk->ds[m] * kx * ky * kz;
                    }
                }
            }
        }
        /* force and velocity update (lbm.cpp:1345-1352) */
#pragma omp parallel for collapse(2)
        for (int k = op->box_lo[2]; k <= op->box_hi[2]; k++)
            for (int j = op->box_lo[1]; j <= op->box_hi[1]; j++)
                for (int i = op->box_lo[0]; i <= op->box_hi[0]; i++) {
                    long c = IDX(o, i, j, k);
                    if (!ibm_node_ok(o->type[c])) continue;
                    long b = (i - op->box_lo[0]) + (long)bx * ((j - op->box_lo[1]) + (long)by * (k - op->box_lo[2]));
                    o->Fx[c] += sgn * Fm[4 * b + 0];
                    o->Fy[c] += sgn * Fm[4 * b + 1];
                    o->Fz[c] += sgn * Fm[4 * b + 2];
                    o->ux[c] += 1.0 * Fm[4 * b + 0] / (2 * o->rho[c]);
                    o->uy[c] += 1.0 * Fm[4 * b + 1] / (2 * o->rho[c]);
                    o->uz[c] += 1.0 * Fm[4 * b + 2] / (2 * o->rho[c]);
                    if (op->thermal) {
                        o->Qh[c] += Fm[4 * b + 3];
                        o->T[c] += 0.5 * Fm[4 * b + 3];
                    }
                }
        /* re-interpolation (lbm.cpp:1362-1387) */
#pragma omp parallel for
        for (int m = 0; m < N; m++) {
            double u3[3];
            interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->ux, o->uy, o->uz, u3);
            mk->ubx[m] = u3[0]; mk->uby[m] = u3[1]; mk->ubz[m] = u3[2];
            if (op->thermal) {
                double t3[3];
                interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->T, NULL, NULL, t3);
                mk->Tb[m] = t3[0];
            }
        }
    }
    free(Fm);
    free(rho_m);
    /* added mass (lbm.cpp:1392-1398) */
    if (op->use_avg_density) {
        double rho = average_density(o, op, mk);
        drag[0] += rho * op->vsolid * (op->vcm_new[0] - op->vcm_old[0]) / 1.0;
        drag[1] += rho * op->vsolid * (op->vcm_new[1] - op->vcm_old[1]) / 1.0;
    }
    force_out[0] = drag[0]; force_out[1] = drag[1]; force_out[2] = drag[2];
    force_out[3] = torque[0]; force_out[4] = torque[1]; force_out[5] = torque[2];
    force_out[6] = heat;
}

/* IBLBM explicit direct forcing (lbm.cpp:1171-1258, Cylinder_IBM branch):
 * unforced rho, u on every F/IN/OUT cell (F kept); the unforced velocity
 * interpolated at the markers; F_m = 2 rho (U_des - U_m) with rho at
 * NearestLatticeCoordinate over [floor x, ceil x] x [floor y, ceil y] x [1, 1];
 * on the box nodes F = sum_m F_m ds_m delta (reset first), u += F / 2 rho and
 * Drag/Lift += -F dx^2 (summed in node order; the reference's OpenMP loop
 * adds them without a reduction).  Then the added mass, as in the implicit
 * scheme.  force_out as orc_ibm_step (torque and heat 0). */
void orc_ibm_step_explicit(orc *o, orc_markers *mk, const orc_ibm_opts *op, double force_out[7]) {
    long n = o->ncell;
    double drag[3] = {0, 0, 0};
#pragma omp parallel for
    for (long c = 0; c < n; c++) {
        if (!ibm_node_ok(o->type[c])) continue;
        double rho = 0, r0 = 0, r1 = 0, r2 = 0;
        for (int l = 0; l < o->q; l++) {
            double fl = o->f[l * n + c];
            rho += fl; r0 += fl * o->cx[l]; r1 += fl * o->cy[l]; r2 += fl * o->cz[l];
        }
        o->rho[c] = rho;
        o->ux[c] = r0 / rho; o->uy[c] = r1 / rho; o->uz[c] = r2 / rho;
    }
    int N = mk->n;
    for (int m = 0; m < N; m++) {
        double u3[3];
        interp3(o, op, mk->x[m], mk->y[m], mk->z[m], o->ux, o->uy, o->uz, u3);
        mk->ubx[m] = u3[0]; mk->uby[m] = u3[1]; mk->ubz[m] = u3[2];
        orc_ibm_opts near = *op;
        near.box_lo[0] = (int)floor(mk->x[m]); near.box_hi[0] = (int)ceil(mk->x[m]);
        near.box_lo[1] = (int)floor(mk->y[m]); near.box_hi[1] = (int)ceil(mk->y[m]);
        near.box_lo[2] = 1; near.box_hi[2] = 1;
        double rho = o->rho[nearest_node(o, &near, mk, m)];
        mk->Fbx[m] = 2 * rho * (mk->udx[m] - mk->ubx[m]) / 1.0;
        mk->Fby[m] = 2 * rho * (mk->udy[m] - mk->uby[m]) / 1.0;
        mk->Fbz[m] = 2 * rho * (mk->udz[m] - mk->ubz[m]) / 1.0;
    }
    for (int i = op->box_lo[0]; i <= op->box_hi[0]; i++)
        for (int j = op->box_lo[1]; j <= op->box_hi[1]; j++)
            for (int k = op->box_lo[2]; k <= op->box_hi[2]; k++) {
                long c = IDX(o, i, j, k);
                if (!ibm_node_ok(o->type[c])) continue;
                double F[3] = {0, 0, 0};
                for (int m = 0; m < N; m++) {
                    double dl = orc_kernel(i - mk->x[m]) * orc_kernel(j - mk->y[m]) * orc_kernel(k - mk->z[m]);
                    F[0] += mk->Fbx[m] * mk->ds[m] * dl;
                    F[1] += mk->Fby[m] * mk->ds[m] * dl;
                    F[2] += mk->Fbz[m] * mk->ds[m] * dl;
                }
                o->Fx[c] = F[0]; o->Fy[c] = F[1]; o->Fz[c] = F[2];
                o->ux[c] += 1.0 * F[0] / (2 * o->rho[c]);
                o->uy[c] += 1.0 * F[1] / (2 * o->rho[c]);
                o->uz[c] += 1.0 * F[2] / (2 * o->rho[c]);
                drag[0] += -F[0] * 1.0;
                drag[1] += -F[1] * 1.0;
            }
    if (op->use_avg_density) {
        double rho = average_density(o, op, mk);
        drag[0] += rho * op->vsolid * (op->vcm_new[0] - op->vcm_old[0]) / 1.0;
        drag[1] += rho * op->vsolid * (op->vcm_new[1] - op->vcm_old[1]) / 1.0;
    }
    force_out[0] = drag[0]; force_out[1] = drag[1]; force_out[2] = drag[2];
    force_out[3] = force_out[4] = force_out[5] = force_out[6] = 0.0;
}

/* One IBM time step in the reference order (main.cpp:197-205):
 * IBLBM -> Collision -> Streaming.  Returns feq<0 count. */
long orc_step_ibm(orc *o, orc_markers *mk, const orc_ibm_opts *op, const double center[3], double force_out[7]) {
    if (op->scheme == 1)
        orc_ibm_step_explicit(o, mk, op, force_out);
    else
        orc_ibm_step(o, mk, op, center, force_out);
    long bad = orc_collide(o);
    orc_stream(o);
    return bad;
}

/* ------------------------------------------------------------------------ */
/* Marker generation and the rigid body (new physics)                        */
/* ------------------------------------------------------------------------ */

/* Fibonacci (golden-angle) sphere of n markers, radius R, centre c; outward
 * normals; area weight pi D^2 / n.  Uses the reference's truncated PI. */
void orc_fibonacci_sphere(int n, double R, const double c[3], double *x, double *y, double *z,
                          double *nx, double *ny, double *nz, double *ds) {
    double ga = REF_PI * (3.0 - sqrt(5.0));
    for (int i = 0; i < n; i++) {
        double zz = 1.0 - (2.0 * i + 1.0) / n;
        double r = sqrt(1.0 - zz * zz);
        double ph = ga * i;
        double ex = r * cos(ph), ey = r * sin(ph), ez = zz;
        x[i] = c[0] + R * ex; y[i] = c[1] + R * ey; z[i] = c[2] + R * ez;
        nx[i] = ex; ny[i] = ey; nz[i] = ez;
        ds[i] = REF_PI * (2 * R) * (2 * R) / n;
    }
}

/* Rigid-body state for a freely moving sphere. */
typedef struct orc_body {
    double xc[3], v[3], om[3];
    double rho_ratio;  /* rho_s / rho_f */
    double vol;        /* V_s */
    double inertia;    /* I_p = 2/5 rho_s V_s R^2 */
    double grav[3];
    int dof;           /* free degrees of freedom: bits 0-2 translation x,y,z, bits 3-5 rotation */
    int have_prev;
    double internal_prev[6];
    double cv;         /* virtual-mass coefficient C_v (0: none) */
    double v_prev[3], om_prev[3];
} orc_body;

/* Fluid momentum and angular momentum inside the body (rho_f = 1), with the
 * volume fraction of node x taken as clamp(R + 1/2 - |x - xc|, 0, 1) and the
 * velocity after the forced collision, u + F/(2 rho) (the whole IBM impulse
 * of this step): out = {sum a u, sum a (x - xc) x u}, over the box in k, j, i
 * order. */
void orc_internal_momentum(orc *o, const double xc[3], double R, const int lo[3], const int hi[3], double out[6]) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int k = lo[2]; k <= hi[2]; k++)
        for (int j = lo[1]; j <= hi[1]; j++)
            for (int i = lo[0]; i <= hi[0]; i++) {
                double rx = i - xc[0], ry = j - xc[1], rz = k - xc[2];
                double a = R + 0.5 - sqrt(rx * rx + ry * ry + rz * rz);
                if (a <= 0) continue;
                if (a > 1) a = 1;
                long c = IDX(o, i, j, k);
                /* momentum after the forced collision: u + F / (2 rho) */
                double hr = 0.5 / o->rho[c];
                double ux = o->ux[c] + hr * o->Fx[c], uy = o->uy[c] + hr * o->Fy[c], uz = o->uz[c] + hr * o->Fz[c];
                s[0] += a * ux; s[1] += a * uy; s[2] += a * uz;
                s[3] += a * (ry * uz - rz * uy);
                s[4] += a * (rz * ux - rx * uz);
                s[5] += a * (rx * uy - ry * ux);
            }
    for (int q = 0; q < 6; q++) out[q] = s[q];
}

/* Newton-Euler step (dt = 1, rho_f = 1) with the internal-fluid treatment of
 * Kempe & Froehlich (J. Comput. Phys. 231, 2012):
 *   rho_s V_s dV/dt   = F_h + d/dt(int u dV) + (rho_s - rho_f) V_s g
 *   I_p dOmega/dt     = T_h + d/dt(int r x u dV)
 * F_h, T_h: reaction of the IBM forces (sum of -F_m ds); the internal terms
 * are differenced between consecutive steps.  With C_v > 0 the virtual-mass
 * scheme of Schwarz, Kempe & Froehlich (J. Comput. Phys. 281, 2015) adds a
 * virtual mass m_v = C_v rho_f V_s (and moment of inertia
 * I_v = C_v 2/5 rho_f V_s R^2) to both sides, the right-hand one lagged a
 * step:
 *   (m + m_v)(V' - V)         = F_h + dI + (rho_s - rho_f) V_s g + m_v (V - V_prev)
 *   (I_p + I_v)(Omega' - Omega) = T_h + dL + I_v (Omega - Omega_prev),
 * which keeps the explicit coupling stable at low density ratios (the
 * smeared forcing drags a shell of outer fluid with the body every step).
 * Degrees of freedom not set in dof keep their velocity.
 * x_c' = x_c + (V + V')/2; markers follow x_c and rotate with Omega'
 * (r' = r + Omega' x r, rescaled to radius R); desired marker velocity
 * V' + Omega' x r'. */
void orc_body_step(orc_body *b, orc_markers *mk, double R, const double force[6], const double internal[6]) {
    if (!b->have_prev) {
        for (int q = 0; q < 6; q++) b->internal_prev[q] = internal[q];
        for (int a = 0; a < 3; a++) {
            b->v_prev[a] = b->v[a];
            b->om_prev[a] = b->om[a];
        }
        b->have_prev = 1;
    }
    const double mass = b->rho_ratio * b->vol;
    const double mv = b->cv * b->vol;
    const double iv = b->cv * b->inertia / b->rho_ratio;
    double vn[3], dxc[3];
    for (int a = 0; a < 3; a++) {
        const double dI = internal[a] - b->internal_prev[a];
        const double dL = internal[3 + a] - b->internal_prev[3 + a];
        const double fb = (mass - b->vol) * b->grav[a];
        vn[a] = ((b->dof >> a) & 1) ? b->v[a] + (force[a] + dI + fb + mv * (b->v[a] - b->v_prev[a])) / (mass + mv)
                                    : b->v[a];
        const double on = ((b->dof >> (3 + a)) & 1)
                              ? b->om[a] + (force[3 + a] + dL + iv * (b->om[a] - b->om_prev[a])) / (b->inertia + iv)
                              : b->om[a];
        b->v_prev[a] = b->v[a];
        b->om_prev[a] = b->om[a];
        b->om[a] = on;
        dxc[a] = 0.5 * (b->v[a] + vn[a]);
        b->xc[a] += dxc[a];
        b->v[a] = vn[a];
    }
    for (int q = 0; q < 6; q++) b->internal_prev[q] = internal[q];
    for (int m = 0; m < mk->n; m++) {
        double r0 = mk->x[m] - (b->xc[0] - dxc[0]);
        double r1 = mk->y[m] - (b->xc[1] - dxc[1]);
        double r2 = mk->z[m] - (b->xc[2] - dxc[2]);
        double q0 = r0 + (b->om[1] * r2 - b->om[2] * r1);
        double q1 = r1 + (b->om[2] * r0 - b->om[0] * r2);
        double q2 = r2 + (b->om[0] * r1 - b->om[1] * r0);
        double s = R / sqrt(q0 * q0 + q1 * q1 + q2 * q2);
        q0 *= s; q1 *= s; q2 *= s;
        mk->x[m] = b->xc[0] + q0; mk->y[m] = b->xc[1] + q1; mk->z[m] = b->xc[2] + q2;
        mk->nx[m] = q0 / R; mk->ny[m] = q1 / R; mk->nz[m] = q2 / R;
        mk->udx[m] = b->v[0] + (b->om[1] * q2 - b->om[2] * q1);
        mk->udy[m] = b->v[1] + (b->om[2] * q0 - b->om[0] * q2);
        mk->udz[m] = b->v[2] + (b->om[0] * q1 - b->om[1] * q0);
    }
}

/* Reference Nusselt number (Find_Nusselt_number, lbm.cpp:3538-3561), summed
 * serially: Nu = 1 + <u_y T>_fluid / (alpha dT / (Ny + 1)). */
double orc_nusselt_volume(orc *o, double alpha, double dT) {
    double s = 0;
    long number = 0;
    for (long c = 0; c < o->ncell; c++) {
        uint8_t t = o->type[c];
        if (t == ORC_F || t == ORC_OUT || t == ORC_IN) { s += o->uy[c] * o->T[c]; number++; }
    }
    return 1 + (s / number) / (alpha * dT / (o->ny + 1));
}
