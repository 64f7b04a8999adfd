// dropin_sphere_bb.cpp -- the reference's staircase-sphere case (Sphere_BB):
// its set-up (main_setup_Sphere / Generate_Sphere, lbm.cpp:1759-1822) and
// time loop with the momentum-exchange coefficients after every step
// (main.cpp:212-221, 365-372), unchanged except for the sizes, through the
// LBM.h facade.
// usage: dropin_sphere_bb NX NY NZ D RE U STEPS OUT.csv [storage 0|1|2]
// Writes "step,cl,cd" rows.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 9) {
        fprintf(stderr, "usage: %s NX NY NZ D RE U STEPS OUT.csv [storage]\n", argv[0]);
        return 2;
    }
    const int Nx = atoi(argv[1]), Ny = atoi(argv[2]), Nz = atoi(argv[3]);
    const double D = atof(argv[4]), Re = atof(argv[5]), u_max = atof(argv[6]);
    const int steps = atoi(argv[7]);
    if (argc > 9) g_lbm_options.storage = atoi(argv[9]);
    const double cs2 = 1.0 / 3.0, nu = u_max * D / Re, tau = 0.5 + nu / cs2;
    const double center_x = Nx / 5.0, center_y = Ny / 2.0, center_z = Nz / 2.0;
    g_lbm_options.u_max = u_max;
    g_lbm_options.ref_area = D * D * PI / 4;  // lbm.cpp:3159-3160
    LBM lb(Nx, Ny, Nz, tau);
    // Generate_Sphere: cells whose centre lies within D/2 of the centre
    for (int i = 1; i <= Nx; i++)
        for (int j = 1; j <= Ny; j++)
            for (int k = 0; k <= Nz; k++) {
                const double rx = i - 0.5, ry = j - 0.5, rz = k - 0.5;
                if (std::sqrt(std::pow(center_x - rx, 2.0) + std::pow(center_y - ry, 2.0) +
                              std::pow(center_z - rz, 2.0)) <= D / 2.0) {
                    lb.fluid[i][j][k].type = TYPE_S;
                    lb.fluid[i][j][k].density = 1.0;
                    lb.fluid[i][j][k].ux = lb.fluid[i][j][k].uy = lb.fluid[i][j][k].uz = 0.0;
                }
            }
    // main_setup_Sphere boundary types and initial state
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int k = 0; k <= Nz + 1; k++) {
                LATTICE &c = lb.fluid[i][j][k];
                if (i == 0) c.type = TYPE_IN;
                if (i == Nx + 1) c.type = TYPE_OUT;
                if (j == 0 || j == Ny + 1) c.type = TYPE_OUT;
                if (k == 0 || k == Nz + 1) c.type = TYPE_OUT;
                if (c.type == TYPE_F || c.type == TYPE_IN || c.type == TYPE_OUT) {
                    c.density = 1.0;
                    c.ux = u_max;
                    c.uy = 0.0;
                    c.uz = 0.0;
                }
            }
    lb.Init();
    FILE *fp = fopen(argv[8], "w");
    if (!fp) return 3;
    fprintf(fp, "step,cl,cd\n");
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
        const double cl = MEA_CL(lb, center_x - D, center_x + D, center_y - D, center_y + D, center_z - D,
                                 center_z + D);
        const double cd = MEA_CD(lb, center_x - D, center_x + D, center_y - D, center_y + D, center_z - D,
                                 center_z + D);
        fprintf(fp, "%d,%.17g,%.17g\n", step, cl, cd);
    }
    fclose(fp);
    printf("{\"steps\": %lld}\n", lb.steps());
    return 0;
}
