// dropin_couette.cpp -- the reference's Couette_Flow build with its ENERGY
// model (#define D2Q9, #define ENERGY): main_setup_Couette (lbm.cpp:1537-1580)
// and the main loop (main.cpp:212-223) through the LBM.h facade built with
// -DD2Q9 -DENERGY.  The constants are those of LBM.h's Couette section
// (LBM.h:206-219), on a strip Nx = 2 wide.
// usage: dropin_couette NY RE STEPS OUT.bin [neumann]
// neumann: the top wall's type_Energy is TYPE_Q (a Neumann wall, j.n = 0).
// Writes, for the interior rows j = 1..Ny of the layer k = 1 (x fastest over
// i = 0..Nx+1, the periodic ghost columns included), as doubles: density, ux,
// uy, uz, T, q[0], q[1], q[2].
#include <cstdio>
#include <cstdlib>
#include <string>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s NY RE STEPS OUT.bin\n", argv[0]);
        return 2;
    }
    const int Nx = 2, Ny = atoi(argv[1]), Nz = 2;
    const double Re = atof(argv[2]);
    const int steps = atoi(argv[3]);
    const bool neumann = argc > 5 && std::string(argv[5]) == "neumann";
    const double cs2 = 1.0 / 3.0, tau = 0.9, rho0 = 1.0;
    const double nu = cs2 * (tau - 0.5);
    const double u_wall = Re * nu / (Ny + 1);
    const double Pr = 0.7, Br = 10, Ec = Br / Pr;
    const double alpha = nu / Pr;
    const double tau_g = 0.5 + alpha / cs2;
    const double k = cs2 * tau_g;
    const double cp = k / (rho0 * alpha);
    const double Tb = 0.5, Tt = Tb + u_wall * u_wall / (cp * Ec);
    g_lbm_options.tau_g = tau_g;
    g_lbm_options.cp = cp;
    g_lbm_options.u_max = u_wall;
    LBM lb(Nx, Ny, Nz, tau);
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int kk = 0; kk <= Nz + 1; kk++) {
                LATTICE &c = lb.fluid[i][j][kk];
                c.type = TYPE_F;
                if (j == 0 || j == Ny + 1) c.type = TYPE_S;
                if (j == Ny + 1) c.ux = u_wall;
                if (j == 0 || j == Ny + 1) {
                    c.type_Energy = (neumann && j == Ny + 1) ? TYPE_Q : TYPE_T;
                    lb.fluid[i][0][kk].T = Tb;
                    lb.fluid[i][Ny + 1][kk].T = Tt;
                }
                if (c.type == TYPE_F) {
                    c.density = 1.0;
                    c.ux = c.uy = c.uz = 0.0;
                    c.T = Tb;
                }
            }
    lb.Init();
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
    }
    lb.sync_to_host();
    FILE *fp = fopen(argv[4], "wb");
    if (!fp) return 3;
    for (int q = 0; q < 8; q++)
        for (int j = 1; j <= Ny; j++)
            for (int i = 0; i <= Nx + 1; i++) {
                const LATTICE &c = lb.fluid[i][j][1];
                const double v[8] = {c.density, c.ux, c.uy, c.uz, c.T, c.q[0], c.q[1], c.q[2]};
                fwrite(&v[q], sizeof(double), 1, fp);
            }
    fclose(fp);
    printf("{\"steps\": %lld}\n", lb.steps());
    return 0;
}
