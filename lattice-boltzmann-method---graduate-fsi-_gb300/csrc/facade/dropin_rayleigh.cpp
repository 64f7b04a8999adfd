// dropin_rayleigh.cpp -- the reference's Rayleigh_Benard build (#define
// ENERGY on D3Q19): main_setup_RayleighBenard1 (lbm.cpp:1585-1643) and the
// main loop with its maximum vertical velocity and Nusselt number every Nt
// = 10 steps, each time rewritten to its two CSV files (main.cpp:212-226,
// 308-321), through the LBM.h facade built with -DENERGY.
// The constants are those of LBM.h's Rayleigh_Benard section
// (LBM.h:222-242) on an NX x NY x NZ box (the reference's is 200 x 50 x 5).
// usage: dropin_rayleigh NX NY NZ STEPS OUT.bin
// Writes, for every cell (ghosts included, x fastest, then y, then z), as
// doubles: density, ux, uy, uz, T, q[0], q[1], q[2]; then the recorded
// maximum |uy| and Nusselt numbers.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s NX NY NZ STEPS OUT.bin\n", argv[0]);
        return 2;
    }
    const int Nx = atoi(argv[1]), Ny = atoi(argv[2]), Nz = atoi(argv[3]), steps = atoi(argv[4]);
    const double cs2 = 1.0 / 3.0, rho0 = 1.0;
    const double Tb = 2, dT = 1, Tt = Tb - dT;
    const double Ra = 1710, g_beta = std::pow(10, -5), Pr = 0.71;
    const double nu = std::sqrt(g_beta * dT * std::pow(Nz + 1, 3) * Pr / Ra);
    const double tau = 0.5 + nu / cs2;
    const double alpha = nu / Pr;
    const double tau_g = 0.5 + alpha / cs2;
    const double k_cond = cs2 * tau_g;
    const double cp = k_cond / (rho0 * alpha);
    const double T_star = (Tb + Tt) / 2;
    g_lbm_options.tau_g = tau_g;
    g_lbm_options.cp = cp;
    g_lbm_options.g_beta = g_beta;
    g_lbm_options.T_star = T_star;
    g_lbm_options.alpha = alpha;
    g_lbm_options.dT = dT;
    const int Nt = 10;
    g_lbm_options.Nt = Nt;
    g_lbm_options.csv_time_step = Nt * 1.0;  // OutputCSV's (i + 1) Nt dt (lbm.cpp:3174-3175)
    LBM lb(Nx, Ny, Nz, tau);
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int k = 0; k <= Nz + 1; k++) {
                LATTICE &c = lb.fluid[i][j][k];
                if (k == 0 || k == Nz + 1 || i == 0 || i == Nx + 1) {
                    c.type = TYPE_S;  // Neumann side walls
                    c.type_Energy = TYPE_Q;
                    c.T = Tt;
                }
                if (j == 0 || j == Ny + 1) {
                    c.type = TYPE_S;  // Dirichlet bottom and top
                    c.type_Energy = TYPE_T;
                    c.T = Tt;
                }
                lb.fluid[i][Ny + 1][k].T = Tb;
                lb.fluid[i][0][k].T = Tt;
                if (c.type == TYPE_F) {
                    c.density = 1.0;
                    c.ux = c.uy = c.uz = 0.0;
                    c.T = Tt;
                    c.F[1] = g_beta * (c.T - T_star);
                }
            }
    lb.Init();
    std::vector<double> uy_max, Nusselt_number;
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
        if (step % Nt == 0) {
            uy_max.push_back(Find_Maximum_uy(lb));
            Nusselt_number.push_back(Find_Nusselt_number(lb));
            std::string name = "Maximum velocity in y direction at Ra = " + std::to_string(Ra) + ".csv";
            OutputCSV(uy_max, name);
            name = "Nusselt number at Ra = " + std::to_string(Ra) + ".csv";
            OutputCSV(Nusselt_number, name);
        }
    }
    lb.sync_to_host();
    FILE *fp = fopen(argv[5], "wb");
    if (!fp) return 3;
    for (int q = 0; q < 8; q++)
        for (int k = 0; k <= Nz + 1; k++)
            for (int j = 0; j <= Ny + 1; j++)
                for (int i = 0; i <= Nx + 1; i++) {
                    const LATTICE &c = lb.fluid[i][j][k];
                    const double v[8] = {c.density, c.ux, c.uy, c.uz, c.T, c.q[0], c.q[1], c.q[2]};
                    fwrite(&v[q], sizeof(double), 1, fp);
                }
    fwrite(uy_max.data(), sizeof(double), uy_max.size(), fp);
    fwrite(Nusselt_number.data(), sizeof(double), Nusselt_number.size(), fp);
    fclose(fp);
    // the per-cell ENERGY helpers on the synced mirror: the bottom wall's T
    // seen from the first fluid cell, and the cell's equilibrium along +y
    const std::vector<double> rest(3, 0.0);
    printf("{\"steps\": %lld, \"uy_max\": %.17g, \"nusselt\": %.17g, \"wall_T_1_1_1\": %.17g, "
           "\"geq_1_1_1_3\": %.17g}\n",
           lb.steps(), uy_max.back(), Nusselt_number.back(), lb.Determine_Wall_Temperature(1, 1, 1),
           lb.Calc_geq(1, 1, 1, 3, TYPE_F, rest));
    return 0;
}
