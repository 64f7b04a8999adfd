// lbm_facade.cpp -- the reference's LBM class surface on top of liblbmgpu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <exception>
#include <string>
#include <vector>

#include "LBM.h"

lbm_options g_lbm_options;

struct lbm_device_state {
    lbm_handle *h = nullptr;
    lbm_energy3d *e3 = nullptr;  // D3Q19 ENERGY builds (-DENERGY without -DD2Q9)
    bool collision_pending = false;
    bool mirror_stale = false;
    bool markers_set = false;
    bool solids = false;      // interior TYPE_S cells on the device
    long long steps = 0;
    std::vector<double> *cl = nullptr, *cd = nullptr;
    int off[3] = {1, 1, 1};  // device cell = reference index - off (0 on periodic axes)
    int dn[3] = {0, 0, 0};
    ~lbm_device_state() {
        if (h) lbmgpu_destroy(h);
        if (e3) lbmgpu_energy3d_destroy(e3);
    }
};

// The reference terminates on invalid state (lbm.cpp:116, 774, 796); the
// facade does the same when the device reports an error.
// the handle whose markers IBLBM registered last (OutputVTK_Marker)
static lbm_handle *g_marker_handle = nullptr;

static void check(const char *what, lbm_status s) {
    if (s != LBM_OK) {
        fprintf(stderr, "lbmgpu %s failed (status %d): %s\n", what, (int)s, lbmgpu_last_error());
        std::terminate();
    }
}

void MARKER::Normal_Marker(int n, double x1, double x2, double y1, double y2, double z1, double z2) {
    (void)n;
    double ddx = x2 - x1, ddy = y2 - y1, ddz = z2 - z1;
    double norm = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
    double t1[3] = {ddx / norm, ddy / norm, ddz / norm};
    const double t2[3] = {0, 0, 1};
    normal[0] = t1[1] * t2[2] - t1[2] * t2[1];
    normal[1] = t1[2] * t2[0] - t1[0] * t2[2];
    normal[2] = t1[0] * t2[1] - t1[1] * t2[0];
}

LBM::LBM(int Nx, int Ny, int Nz, double tau) : Nx(Nx), Ny(Ny), Nz(Nz), tau(tau) {
    dev = std::make_shared<lbm_device_state>();
    fluid = new LATTICE **[Nx + 2];
    for (int i = 0; i < Nx + 2; i++) {
        fluid[i] = new LATTICE *[Ny + 2];
        for (int j = 0; j < Ny + 2; j++) fluid[i][j] = new LATTICE[Nz + 2];
    }
}

int LBM::getNx() const { return Nx; }
int LBM::getNy() const { return Ny; }
int LBM::getNz() const { return Nz; }
double LBM::getTAU() const { return tau; }
lbm_handle *LBM::handle() const { return dev->h; }
lbm_energy3d *LBM::energy3d() const { return dev->e3; }
long long LBM::steps() const { return dev->steps; }

double LBM::Calc_feq(int i, int j, int k, int l) {
    const LATTICE &c = fluid[i][j][k];
    const double cs2 = 1.0 / 3.0;
    double u_dot_u = c.ux * c.ux + c.uy * c.uy + c.uz * c.uz;
    double c_dot_u = c.ux * cx[l] + c.uy * cy[l] + c.uz * cz[l];
    return c.density * w[l] *
           (1 + c_dot_u / cs2 + c_dot_u * c_dot_u / (2 * cs2 * cs2) - u_dot_u / (2 * cs2) +
            std::pow(c_dot_u, 3) / (6 * std::pow(cs2, 3)) - c_dot_u * u_dot_u / (2 * cs2 * cs2));
}

void LBM::ConvLBM(int i, int j, int k) {
    LATTICE &c = fluid[i][j][k];
    const double omega = 1.0 / tau, cs2 = 1.0 / 3.0;
    double F_dot_u = c.F[0] * c.ux + c.F[1] * c.uy + c.F[2] * c.uz;
    for (int l = 0; l < npop; l++) {
        double c_dot_u = c.ux * cx[l] + c.uy * cy[l] + c.uz * cz[l];
        double f_eq = Calc_feq(i, j, k, l);
        double F_dot_c = c.F[0] * cx[l] + c.F[1] * cy[l] + c.F[2] * cz[l];
        double S = (1 - omega * 0.5) * w[l] * (F_dot_c / cs2 + F_dot_c * c_dot_u / (cs2 * cs2) - F_dot_u / cs2);
        c.f_star[l] = c.f[l] * (1 - omega) + omega * f_eq + S;
    }
}

void LBM::Determine_Wall_Velocity(int i, int j, int k, std::vector<double> &uwall) {
    int num = 0;
    for (int l = 0; l < npop; l++) {
        int in = (i + cx[l] + (Nx + 2)) % (Nx + 2), jn = (j + cy[l] + (Ny + 2)) % (Ny + 2),
            kn = (k + cz[l] + (Nz + 2)) % (Nz + 2);
        const LATTICE &nb = fluid[in][jn][kn];
        if (nb.type == TYPE_S && (nb.ux != 0 || nb.uy != 0 || nb.uz != 0)) {
            uwall[0] += nb.ux;
            uwall[1] += nb.uy;
            uwall[2] += nb.uz;
            num++;
        }
    }
    if (num) {
        uwall[0] /= num;
        uwall[1] /= num;
        uwall[2] /= num;
    }
}

#if defined ENERGY
// rho w T times the cubic shape of c.u: the cell's own T and u, or for a
// solid type the wall T of the cell and the given wall velocity
double LBM::Calc_geq(int i, int j, int k, int l, short type, std::vector<double> uwall) {
    const LATTICE &c = fluid[i][j][k];
    const double cs2 = 1.0 / 3.0;
    double T = c.T, u[3] = {c.ux, c.uy, c.uz};
    if (type == TYPE_S) {
        T = Determine_Wall_Temperature(i, j, k);
        for (int a = 0; a < 3; a++) u[a] = uwall[a];
    }
    const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double cu = u[0] * cx[l] + u[1] * cy[l] + u[2] * cz[l];
    return c.density * w[l] * T *
           (1 + cu / cs2 + cu * cu / (2 * cs2 * cs2) - uu / (2 * cs2) + std::pow(cu, 3) / (6 * std::pow(cs2, 3)) -
            cu * uu / (2 * cs2 * cs2));
}

// the mean T of the solid neighbours (periodic modulo over the whole grid)
double LBM::Determine_Wall_Temperature(int i, int j, int k) {
    double s = 0.0;
    int num = 0;
    for (int l = 0; l < npop; l++) {
        const LATTICE &nb = fluid[(i + cx[l] + Nx + 2) % (Nx + 2)][(j + cy[l] + Ny + 2) % (Ny + 2)]
                                 [(k + cz[l] + Nz + 2) % (Nz + 2)];
        if (nb.type == TYPE_S) {
            s += nb.T;
            num++;
        }
    }
    return s / num;
}

// T_w = (j.n - sum over the links facing away from the walls of g c.n) /
// sum over the wall links of geq(rho, T = 1, u_w) c.n, n the mean wall-link
// direction (not normalised)
double LBM::Determine_Twall_Neumann(int i, int j, int k, std::vector<double> uwall, std::vector<int> cdotn_pos,
                                   std::vector<int> cdotn_notpos, double j_dot_n) {
    const LATTICE &c = fluid[i][j][k];
    const double cs2 = 1.0 / 3.0;
    double n[3] = {0, 0, 0};
    for (int l : cdotn_pos) {
        n[0] += cx[l];
        n[1] += cy[l];
        n[2] += cz[l];
    }
    for (int a = 0; a < 3; a++) n[a] /= (double)cdotn_pos.size();
    double other = 0.0;
    for (int l : cdotn_notpos) other += c.g[l] * (cx[l] * n[0] + cy[l] * n[1] + cz[l] * n[2]);
    const double uu = uwall[0] * uwall[0] + uwall[1] * uwall[1] + uwall[2] * uwall[2];
    double wall = 0.0;
    for (int l : cdotn_pos) {
        const double cu = uwall[0] * cx[l] + uwall[1] * cy[l] + uwall[2] * cz[l];
        const double eq = w[l] * c.density *
                          (1 + cu / cs2 + cu * cu / (2 * cs2 * cs2) - uu / (2 * cs2) +
                           std::pow(cu, 3) / (6 * std::pow(cs2, 3)) - cu * uu / (2 * cs2 * cs2));
        wall += eq * (cx[l] * n[0] + cy[l] * n[1] + cz[l] * n[2]);
    }
    const double Tw = (j_dot_n - other) / wall;
    for (int l = 0; l < npop; l++) {
        const int o = opposite[l];
        if (cx[o] == n[0] && cy[o] == n[1] && cz[o] == n[2]) {
            fluid[(i + cx[l] + Nx + 2) % (Nx + 2)][(j + cy[l] + Ny + 2) % (Ny + 2)][(k + cz[l] + Nz + 2) % (Nz + 2)]
                .T = Tw;
            break;
        }
    }
    return Tw;
}
#endif

#if defined ENERGY && !defined D2Q9
// D3Q19 with ENERGY (the reference's Rayleigh_Benard build): the whole
// ghost-inclusive set-up goes to lbmgpu_energy3d, which keeps the
// reference's grid.
static void init_energy3d(LBM &lb, lbm_device_state &d, double tau) {
    const int Nx = lb.getNx(), Ny = lb.getNy(), Nz = lb.getNz();
    const int NX = Nx + 2, NY = Ny + 2, NZ = Nz + 2;
    const size_t n = (size_t)NX * NY * NZ;
    std::vector<uint8_t> t(n), te(n);
    std::vector<double> T(n), rho(n), u(3 * n), F(3 * n);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) {
                const LATTICE &c = lb.fluid[i][j][k];
                const size_t id = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k);
                t[id] = (uint8_t)c.type;
                te[id] = (uint8_t)c.type_Energy;
                T[id] = c.T;
                rho[id] = c.density;
                u[id] = c.ux;
                u[n + id] = c.uy;
                u[2 * n + id] = c.uz;
                for (int a = 0; a < 3; a++) F[a * n + id] = c.F[a];
            }
    const lbm_options &o = g_lbm_options;
    lbm_energy3d_setup su = {};
    su.nx = Nx;
    su.ny = Ny;
    su.nz = Nz;
    su.tau = tau;
    su.tau_g = o.tau_g;
    su.cp = o.cp;
    su.g_beta = o.g_beta;
    su.T_star = o.T_star;
    su.type = t.data();
    su.type_energy = te.data();
    su.T = T.data();
    su.rho = rho.data();
    su.u = u.data();
    su.F = F.data();
    if (d.e3) lbmgpu_energy3d_destroy(d.e3);
    d.e3 = nullptr;
    check("energy3d_create", lbmgpu_energy3d_create(&su, &d.e3));
}
#endif

void LBM::Init() {
    const int NX = Nx + 2, NY = Ny + 2, NZ = Nz + 2;
    const size_t n = (size_t)NX * NY * NZ;
#if defined ENERGY && !defined D2Q9
    (void)n;
    init_energy3d(*this, *dev, tau);
    // host mirror as LBM::Init leaves it (lbm.cpp:31-57): f = feq, g = geq of
    // the cell type with the walls at rest
    const std::vector<double> rest(3, 0.0);
    for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++)
            for (int k = 0; k < NZ; k++)
                for (int l = 0; l < npop; l++) {
                    double fe = Calc_feq(i, j, k, l);
                    fluid[i][j][k].f[l] = fe;
                    fluid[i][j][k].f_star[l] = fe;
                    double ge = Calc_geq(i, j, k, l, fluid[i][j][k].type, rest);
                    fluid[i][j][k].g[l] = ge;
                    fluid[i][j][k].g_star[l] = ge;
                }
    dev->steps = 0;
    dev->mirror_stale = false;
    return;
#endif
    std::vector<uint8_t> types(n);
    std::vector<double> rho(n), ux(n), uy(n), uz(n), T(n);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) {
                const LATTICE &c = fluid[i][j][k];
                size_t id = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k);
                types[id] = (uint8_t)c.type;
                rho[id] = c.density;
                ux[id] = c.ux;
                uy[id] = c.uy;
                uz[id] = c.uz;
                T[id] = c.T;
            }
    lbm_config cfg;
#if defined D2Q9
    // the computational layer k = 1 (the k = 0, 2 layers of a D2Q9 build
    // evolve on their own and are never read)
    {
        const size_t layer = (size_t)NX * NY;
        check("config_from_types_2d",
              lbmgpu_config_from_types_2d(Nx, Ny, tau, types.data() + layer, rho.data() + layer, ux.data() + layer,
                                          uy.data() + layer, &cfg));
    }
#else
    check("config_from_types", lbmgpu_config_from_types(Nx, Ny, Nz, tau, types.data(), rho.data(), ux.data(),
                                                        uy.data(), uz.data(), T.data(), &cfg));
#endif
    const lbm_options &o = g_lbm_options;
    // a uniform force on the fluid cells of the set-up (main_setup_Poiseuille
    // writes F[0] = -dp_dx, lbm.cpp:1518) is the body force of the run
    {
        bool have = false, uniform = true;
        double F0[3] = {0, 0, 0};
        for (int i = 0; i < NX; i++)
            for (int j = 0; j < NY; j++)
                for (int k = 0; k < NZ; k++) {
                    const LATTICE &c = fluid[i][j][k];
                    if (c.type != TYPE_F) continue;
                    if (!have) {
                        for (int a = 0; a < 3; a++) F0[a] = c.F[a];
                        have = true;
                    } else if (c.F[0] != F0[0] || c.F[1] != F0[1] || c.F[2] != F0[2]) {
                        uniform = false;
                    }
                }
        if (have && uniform && (F0[0] != 0 || F0[1] != 0 || F0[2] != 0))
            for (int a = 0; a < 3; a++) cfg.body_force[a] = F0[a];
    }
    cfg.wall_force = o.wall_force;
    cfg.storage = o.storage;
    cfg.thermal = o.thermal;
    cfg.tau_g = o.tau_g;
    cfg.T_ref = o.T_ref;
    for (int a = 0; a < 3; a++) cfg.gbeta[a] = o.gbeta[a];
#if defined ENERGY && defined D2Q9
    // the energy set-up of main_setup_Couette (lbm.cpp:1552-1572):
    // type_Energy and T of the computational layer
    {
        const size_t layer = (size_t)NX * NY;
        std::vector<uint8_t> te((size_t)NX * NY);
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) te[(size_t)i + (size_t)NX * j] = (uint8_t)fluid[i][j][1].type_Energy;
        check("config_energy_2d", lbmgpu_config_energy_2d(&cfg, Nx, Ny, types.data() + layer, te.data(),
                                                          T.data() + layer, o.tau_g, o.cp));
    }
#endif
    const int dims[3] = {Nx, Ny, Nz};
    const int ddims[3] = {cfg.nx, cfg.ny, cfg.nz};
    for (int a = 0; a < 3; a++) {
        dev->off[a] = ddims[a] == dims[a] + 2 ? 0 : 1;
        dev->dn[a] = ddims[a];
    }
#if defined D2Q9
    dev->off[2] = 1;  // device layer 0 is the reference's k = 1
    dev->dn[2] = 1;
#endif
    if (dev->h) lbmgpu_destroy(dev->h);
    dev->h = nullptr;
    check("create", lbmgpu_create(&cfg, &dev->h));
    const size_t nd = (size_t)cfg.nx * cfg.ny * cfg.nz;
    // interior TYPE_S cells (Generate_Sphere and the like): solid mask
    {
        std::vector<uint8_t> mask(nd, 0);
        bool any = false;
        for (int z = 0; z < cfg.nz; z++)
            for (int y = 0; y < cfg.ny; y++)
                for (int x = 0; x < cfg.nx; x++) {
                    const int i = x + dev->off[0], j = y + dev->off[1], k = z + dev->off[2];
                    const bool ghost = (dev->off[0] && (i == 0 || i == Nx + 1)) ||
                                       (dev->off[1] && (j == 0 || j == Ny + 1)) ||
                                       (dev->off[2] && (k == 0 || k == Nz + 1));
                    if (!ghost && fluid[i][j][k].type == TYPE_S) {
                        mask[(size_t)x + (size_t)cfg.nx * ((size_t)y + (size_t)cfg.ny * z)] = 1;
                        any = true;
                    }
                }
        if (any) check("set_solids", lbmgpu_set_solids(dev->h, mask.data()));
        dev->solids = any;
    }
#if defined MORE_DETAILS
    check("set_more_details", lbmgpu_set_more_details(dev->h, 1));
#endif
    std::vector<double> drho(nd), dux(nd), duy(nd), duz(nd), dT(nd);
    for (int z = 0; z < cfg.nz; z++)
        for (int y = 0; y < cfg.ny; y++)
            for (int x = 0; x < cfg.nx; x++) {
                const LATTICE &c = fluid[x + dev->off[0]][y + dev->off[1]][z + dev->off[2]];
                size_t id = (size_t)x + (size_t)cfg.nx * ((size_t)y + (size_t)cfg.ny * z);
                drho[id] = c.density;
                dux[id] = c.ux;
                duy[id] = c.uy;
                duz[id] = c.uz;
                dT[id] = c.T;
            }
    check("init_fields", lbmgpu_init_fields(dev->h, drho.data(), dux.data(), duy.data(), duz.data(),
                                            cfg.thermal ? dT.data() : nullptr));
    // host mirror as LBM::Init leaves it (lbm.cpp:31-57)
    for (int i = 0; i < NX; i++)
        for (int j = 0; j < NY; j++)
            for (int k = 0; k < NZ; k++)
                for (int l = 0; l < npop; l++) {
                    double fe = Calc_feq(i, j, k, l);
                    fluid[i][j][k].f[l] = fe;
                    fluid[i][j][k].f_star[l] = fe;
                }
    dev->steps = 0;
    dev->mirror_stale = false;
}

void LBM::Collision() { dev->collision_pending = true; }

void LBM::Streaming() {
    if (dev->e3) {
        check("energy3d_step", lbmgpu_energy3d_step(dev->e3, 1));
        dev->collision_pending = false;
        dev->mirror_stale = true;
        dev->steps++;
        return;
    }
    if (!dev->h) check("Streaming before Init", LBM_ERR_STATE);
    check("step", lbmgpu_step(dev->h, 1));
    dev->collision_pending = false;
    dev->mirror_stale = true;
    dev->steps++;
    if (dev->markers_set && dev->cl && dev->cd) {
        double f[8];
        int got = 0;
        check("get_forces", lbmgpu_get_forces(dev->h, f, 1, &got));
        const lbm_options &o = g_lbm_options;
        const double q = 0.5 * o.rho0 * o.u_max * o.u_max * o.ref_area;
        dev->cd->push_back(f[0] / q);
        dev->cl->push_back(f[1] / q);
    }
}

void LBM::MacroProp() { dev->mirror_stale = true; }

void LBM::sync_to_host() {
    if (dev->e3) {
        // every cell, ghosts included (the walls as MacroProp leaves them)
        const int NX = Nx + 2, NY = Ny + 2, NZ = Nz + 2;
        const size_t n = (size_t)NX * NY * NZ;
        std::vector<double> v(8 * n);
        for (int f = 0; f < 8; f++)
            check("energy3d_download", lbmgpu_energy3d_download(dev->e3, f, v.data() + (size_t)f * n));
        for (int k = 0; k < NZ; k++)
            for (int j = 0; j < NY; j++)
                for (int i = 0; i < NX; i++) {
                    const size_t id = (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k);
                    LATTICE &c = fluid[i][j][k];
                    c.density = v[id];
                    c.ux = v[n + id];
                    c.uy = v[2 * n + id];
                    c.uz = v[3 * n + id];
                    c.T = v[4 * n + id];
#if defined ENERGY
                    for (int a = 0; a < 3; a++) c.q[a] = v[(5 + a) * n + id];
#endif
                }
        dev->mirror_stale = false;
        return;
    }
    if (!dev->h) return;
    const size_t nd = (size_t)dev->dn[0] * dev->dn[1] * dev->dn[2];
#if defined ENERGY
    const int nf = 5;
    std::vector<float> qx(nd), qy(nd);
    check("download", lbmgpu_download_f32(dev->h, LBM_FIELD_QX, qx.data()));
    check("download", lbmgpu_download_f32(dev->h, LBM_FIELD_QY, qy.data()));
#else
    const int nf = g_lbm_options.thermal ? 5 : 4;
#endif
    std::vector<float> buf(nf * nd);
    check("download", lbmgpu_download_all_f32(dev->h, buf.data()));
    for (int z = 0; z < dev->dn[2]; z++)
        for (int y = 0; y < dev->dn[1]; y++)
            for (int x = 0; x < dev->dn[0]; x++) {
                size_t id = (size_t)x + (size_t)dev->dn[0] * ((size_t)y + (size_t)dev->dn[1] * z);
                LATTICE &c = fluid[x + dev->off[0]][y + dev->off[1]][z + dev->off[2]];
                c.density = buf[id];
                c.ux = buf[nd + id];
                c.uy = buf[2 * nd + id];
                c.uz = buf[3 * nd + id];
                if (nf == 5) c.T = buf[4 * nd + id];
#if defined ENERGY
                c.q[0] = qx[id];
                c.q[1] = qy[id];
                c.q[2] = 0.0;
#endif
            }
#if defined MORE_DETAILS
    std::vector<float> det(LBM_DETAIL_COUNT * nd);
    std::vector<double> st(LBM_STAT_COUNT * nd);
    check("download_details", lbmgpu_download_details(dev->h, det.data()));
    check("download_stats", lbmgpu_download_stats(dev->h, st.data(), nullptr, nullptr));
    static const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    for (int z = 0; z < dev->dn[2]; z++)
        for (int y = 0; y < dev->dn[1]; y++)
            for (int x = 0; x < dev->dn[0]; x++) {
                size_t id = (size_t)x + (size_t)dev->dn[0] * ((size_t)y + (size_t)dev->dn[1] * z);
                LATTICE &c = fluid[x + dev->off[0]][y + dev->off[1]][z + dev->off[2]];
                c.pressure = det[id];
                c.avg_pressure = st[LBM_STAT_AVG_P * nd + id];
                c.rms_pressure = st[LBM_STAT_RMS_P * nd + id];
                for (int a = 0; a < 3; a++) {
                    c.avg_velocity[a] = st[(LBM_STAT_AVG_U + a) * nd + id];
                    c.rms_velocity[a] = st[(LBM_STAT_RMS_U + a) * nd + id];
                }
                for (int q = 0; q < 6; q++) {
                    const int a = ia[q], b = ib[q];
                    c.sigma[a][b] = c.sigma[b][a] = det[(LBM_DETAIL_SXX + q) * nd + id];
                    c.avg_ReynoldStress[a][b] = c.avg_ReynoldStress[b][a] = st[(LBM_STAT_AVG_RS + q) * nd + id];
                    c.rms_ReynoldStress[a][b] = c.rms_ReynoldStress[b][a] = st[(LBM_STAT_RMS_RS + q) * nd + id];
                }
            }
#endif
    dev->mirror_stale = false;
}

#if defined MORE_DETAILS
void LBM::Sup_MacroProp(int n) {
    if (!dev->h) check("Sup_MacroProp before Init", LBM_ERR_STATE);
    check("sup_macroprop", lbmgpu_sup_macroprop(dev->h, n, g_lbm_options.Nt, 1.0));
    dev->mirror_stale = true;
}
#endif

double kernel(double r) {
    double a = std::fabs(r);
    if (a <= 1) return (3 - 2 * a + std::sqrt(1 + 4 * a - 4 * r * r)) / 8;
    if (a <= 2) return (5 - 2 * a - std::sqrt(-7 + 12 * a - 4 * r * r)) / 8;
    return 0;
}

void NearestLatticeCoordinate(int xmin, int xmax, int ymin, int ymax, int zmin, int zmax, int &i, int &j, int &k,
                              std::vector<MARKER> &marker, int n) {
    double dot = 0;
    for (int x = xmin; x <= xmax; x++)
        for (int y = ymin; y <= ymax; y++)
            for (int z = zmin; z <= zmax; z++) {
                double d = (x - marker[n].x) * marker[n].normal[0] + (y - marker[n].y) * marker[n].normal[1] +
                           (z - marker[n].z) * marker[n].normal[2];
                if (d >= dot && d > 0) {
                    i = x;
                    j = y;
                    k = z;
                    dot = d;
                }
            }
}

double Calc_AverageDensity(LBM &lb, std::vector<MARKER> &marker, int xmin, int xmax, int ymin, int ymax, int zmin,
                           int zmax) {
    double rho = 0;
    int number = 0;
    for (int i = xmin; i <= xmax; i++)
        for (int j = ymin; j <= ymax; j++)
            for (int k = zmin; k <= zmax; k++) {
                bool inside = true;
                for (size_t n = 0; n < marker.size() && inside; n++) {
                    double d = (i - marker[n].x) * marker[n].normal[0] + (j - marker[n].y) * marker[n].normal[1] +
                               (k - marker[n].z) * marker[n].normal[2];
                    if (d > 0) inside = false;
                }
                if (inside) {
                    rho += lb.fluid[i][j][k].density;
                    number++;
                }
            }
    return number ? rho / number : 0.0;
}

void IBLBM(LBM &lb, std::vector<MARKER> &marker, std::vector<double> &ds, std::vector<double> &Cl,
           std::vector<double> &Cd, double V_CM[], double t) {
    (void)t;
    lbm_device_state &d = *lb.dev;
    if (!d.h) check("IBLBM before Init", LBM_ERR_STATE);
    d.cl = &Cl;
    d.cd = &Cd;
    // the markers stay on the device (a prescribed D2Q9 motion moves them
    // there: lbmgpu_get_markers reads them back)
    if (d.markers_set) {
        g_marker_handle = d.h;
        return;
    }
    const int n = (int)marker.size();
    std::vector<double> xyz(3 * (size_t)n), dsv(ds.begin(), ds.end());
    double c[3] = {0, 0, 0};
    for (int m = 0; m < n; m++) {
        // device node coordinates: reference index minus the device offset
        xyz[m] = marker[m].x - (d.off[0] - 1);
        xyz[n + m] = marker[m].y - (d.off[1] - 1);
        xyz[2 * (size_t)n + m] = marker[m].z - (d.off[2] - 1);
        for (int a = 0; a < 3; a++) c[a] += xyz[(size_t)a * n + m] / n;
    }
    const lbm_options &o = g_lbm_options;
    if (o.body_center_set)
        for (int a = 0; a < 3; a++) c[a] = o.body_center[a] - (d.off[a] - 1);
    double R = o.body_radius;
    if (R <= 0)
        for (int m = 0; m < n; m++) {
            double rr = 0;
            for (int a = 0; a < 3; a++) rr += (xyz[(size_t)a * n + m] - c[a]) * (xyz[(size_t)a * n + m] - c[a]);
            R = std::max(R, std::sqrt(rr));
        }
    lbm_ibm_config ic = {};
    ic.n_markers = n;
    ic.m_max = o.m_max;
    ic.literal_sign = o.literal_sign;
    ic.radius = R;
    for (int a = 0; a < 3; a++) {
        ic.center[a] = c[a];
        ic.velocity[a] = V_CM[a];
    }
#if defined D2Q9
    // V_CM(t) is prescribed on the device; V_CM[] is the reference's initial zero
    for (int a = 0; a < 3; a++) ic.velocity[a] = o.motion_velocity[a];
    ic.rho_nearest = o.rho_nearest;
    ic.added_mass = o.added_mass;
    ic.volume = o.vsolid;
    ic.motion = o.motion;
    ic.motion_amp = o.motion_amp;
    ic.motion_freq = o.motion_freq;
    ic.scheme = o.ibm_scheme;
#endif
    check("set_markers", lbmgpu_set_markers(d.h, &ic, xyz.data(), dsv.data(), nullptr));
#if defined D2Q9
    std::vector<double> nrm(3 * (size_t)n);
    for (int m = 0; m < n; m++)
        for (int a = 0; a < 3; a++) nrm[(size_t)a * n + m] = marker[m].normal[a];
    check("set_marker_normals", lbmgpu_set_marker_normals(d.h, nrm.data()));
#endif
    d.markers_set = true;
    g_marker_handle = d.h;
}

// Momentum-exchange coefficients of the solid cells after the latest step
// (MEA_CL / MEA_CD, lbm.cpp:3085-3163).  A D3Q19 build sums over every
// fluid cell next to an interior solid after every step (one body; the
// reference's box only keeps the domain walls out of the sum).  A D2Q9 build
// sums over the given box of the current state, so each body of the tandem
// cases keeps its own coefficients.
static double mea_component(LBM &lb, int comp, const int box[6]) {
    lbm_handle *h = lb.handle();
    if (!h) return 0.0;
    const lbm_options &o = g_lbm_options;
    const double q = 0.5 * o.rho0 * o.u_max * o.u_max * o.ref_area;
#if defined D2Q9
    double F[3];
    check("mea_box", lbmgpu_mea_box(h, box, F));
    return F[comp] / q;
#else
    (void)box;
    std::vector<double> rows(4);
    int n = 0;
    if (lbmgpu_get_solid_forces(h, rows.data(), 1, &n) != LBM_OK || n < 1) return 0.0;
    return rows[comp] / q;
#endif
}

double MEA_CL(LBM &lb, int xmin, int xmax, int ymin, int ymax, int zmin, int zmax) {
    const int box[6] = {xmin, xmax, ymin, ymax, zmin, zmax};
    return -mea_component(lb, 1, box);
}
double MEA_CD(LBM &lb, int xmin, int xmax, int ymin, int ymax, int zmin, int zmax) {
    const int box[6] = {xmin, xmax, ymin, ymax, zmin, zmax};
    return mea_component(lb, 0, box);
}

// OutputVTK (lbm.cpp:2290-2642) without the host mirror: the device writes
// ./field%06d.vtr of the current state from a host thread while the time
// loop goes on.  Velocity is divided by g_lbm_options.u_max as the reference
// does; the cell types come from fluid[..].type.
// fluid[..].type for the CellType array: every layer, or the layer k = 1 of
// a D2Q9 build
static std::vector<uint8_t> cell_types(LBM &lb) {
    const int NX = lb.getNx() + 2, NY = lb.getNy() + 2;
#if defined D2Q9
    const int k0 = 1, NZ = 1;
#else
    const int k0 = 0, NZ = lb.getNz() + 2;
#endif
    std::vector<uint8_t> types((size_t)NX * NY * NZ);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++)
                types[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)] = (uint8_t)lb.fluid[i][j][k0 + k].type;
    return types;
}

void OutputVTK_async(int &nout, LBM &lb) {
    lbm_handle *h = lb.handle();
    if (!h) check("OutputVTK_async before Init", LBM_ERR_STATE);
    const std::vector<uint8_t> types = cell_types(lb);
    char name[64];
    snprintf(name, sizeof(name), "./field%06d.vtr", nout);
    check("output_vtk_async", lbmgpu_output_vtk_async(h, name, g_lbm_options.u_max, types.data()));
}

void OutputVTK(int &nout, LBM &lb) {
    OutputVTK_async(nout, lb);
    check("output_wait", lbmgpu_output_wait(lb.handle()));
}

void OutputVTK_Marker(int &time, std::vector<MARKER> &marker) {
    char name[64];
    snprintf(name, sizeof(name), "wall_t %d.vtk", time / std::max(1, g_lbm_options.Nt));
    if (g_marker_handle) {
        check("output_markers_vtk", lbmgpu_output_markers_vtk(g_marker_handle, name));
        return;
    }
    // before IBLBM: the caller's set-up positions, in the same format
    FILE *fp = fopen(name, "w");
    if (!fp) check("OutputVTK_Marker: cannot open the file", LBM_ERR_INVALID);
    const int n = (int)marker.size();
    fprintf(fp, "# vtk DataFile Version 3.0\nwall_state\nASCII\nDATASET POLYDATA\n");
    fprintf(fp, "POINTS %d float\n", n);
    for (int m = 0; m < n; m++) fprintf(fp, "%g %g %g \n", marker[m].x, marker[m].y, marker[m].z);
    fprintf(fp, "LINES %d %d\n", n, 3 * n);
    for (int m = 0; m < n; m++) fprintf(fp, "2 %d %d\n", m % n, (m + 1) % n);
    fprintf(fp, "VERTICES 1 %d\n", n + 1);
    fprintf(fp, "%d ", n);
    for (int m = 0; m < n; m++) fprintf(fp, "%d ", m);
    fclose(fp);
}

void OutputCSV(std::vector<double> &error, std::string name) {
    check("output_csv", lbmgpu_output_csv(name.c_str(), error.data(), (int)error.size(), g_lbm_options.csv_time_step));
}

double Find_Nusselt_number(LBM &lb) {
    if (lb.energy3d()) {
        // lbm.cpp:3538-3561 on the mirror, summed in the serial order
        lb.sync_to_host();
        double s = 0.0;
        long long number = 0;
        for (int i = 0; i <= lb.getNx() + 1; i++)
            for (int j = 0; j <= lb.getNy() + 1; j++)
                for (int k = 0; k <= lb.getNz() + 1; k++) {
                    const LATTICE &c = lb.fluid[i][j][k];
                    if (c.type == TYPE_F || c.type == TYPE_OUT || c.type == TYPE_IN) {
                        s += c.uy * c.T;
                        number++;
                    }
                }
        return 1 + (s / number) / (g_lbm_options.alpha * g_lbm_options.dT / (lb.getNy() + 1));
    }
    lbm_handle *h = lb.handle();
    if (!h) check("Find_Nusselt_number before Init", LBM_ERR_STATE);
    double nu = 0.0;
    check("nusselt", lbmgpu_nusselt(h, g_lbm_options.alpha, g_lbm_options.dT, &nu));
    return nu;
}

// Find_Maximum_uy (lbm.cpp:3522-3536): max |u_y| over every cell, ghosts
// included, of the current moments
double Find_Maximum_uy(LBM &lb) {
    lb.sync_to_host();
    double maximum = -99;
    for (int i = 0; i <= lb.getNx() + 1; i++)
        for (int j = 0; j <= lb.getNy() + 1; j++)
            for (int k = 0; k <= lb.getNz() + 1; k++) maximum = std::max(maximum, std::fabs(lb.fluid[i][j][k].uy));
    return maximum;
}

#if defined MORE_DETAILS
// OutputAVGVTK: the reference names its file only for its tandem-triangle
// case (lbm.cpp:2654-2658); here it is always ./avgfield.vtr.
void OutputAVGVTK(int &, LBM &lb) {
    lbm_handle *h = lb.handle();
    if (!h) check("OutputAVGVTK before Init", LBM_ERR_STATE);
    const int NX = lb.getNx() + 2, NY = lb.getNy() + 2, NZ = lb.getNz() + 2;
    std::vector<uint8_t> types((size_t)NX * NY * NZ);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++)
                types[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)] = (uint8_t)lb.fluid[i][j][k].type;
    check("output_avg_vtk", lbmgpu_output_avg_vtk(h, "./avgfield.vtr", g_lbm_options.u_max, types.data()));
}
#endif
