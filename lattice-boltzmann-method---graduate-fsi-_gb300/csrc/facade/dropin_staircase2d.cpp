// dropin_staircase2d.cpp -- the reference's staircase 2D cases with the
// momentum-exchange algorithm (#define D2Q9, MOMENTUM_EXCHANGE_ALGORITHM):
// Cylinder_Basic (main_setup_Cylinder, lbm.cpp:1429-1494), Cylinder_Tandem_
// Circle (lbm.cpp:1645-1704) and Cylinder_Tandem_Triangle (lbm.cpp:1706-
// 1757), set up as the reference does and run by its loop (main.cpp:212-223)
// through the LBM.h facade built with -DD2Q9; MEA_CL / MEA_CD of every body
// in its box (main.cpp:242-356), taken after every step here.
// usage: dropin_staircase2d KIND NX NY D RE U LPD NB STEPS OUT.bin
//   KIND: cylbasic | tandem | triangle
// Writes, as doubles: Cl[body][step], then Cd[body][step].
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 11) {
        fprintf(stderr, "usage: %s KIND NX NY D RE U LPD NB STEPS OUT.bin\n", argv[0]);
        return 2;
    }
    const char *kind = argv[1];
    const int Nx = atoi(argv[2]), Ny = atoi(argv[3]), Nz = 1;
    const double Dd = atof(argv[4]), Re = atof(argv[5]), u_max = atof(argv[6]), LpD = atof(argv[7]);
    const int NB = atoi(argv[8]), steps = atoi(argv[9]);
    const double cs2 = 1.0 / 3.0;
    const double nu = u_max * Dd / Re;
    const double tau = 0.5 + nu / cs2;
    g_lbm_options.u_max = u_max;
    LBM lb(Nx, Ny, Nz, tau);
    std::vector<std::array<int, 4>> boxes;
    const bool basic = !strcmp(kind, "cylbasic"), tandem = !strcmp(kind, "tandem"), tri = !strcmp(kind, "triangle");
    if (!basic && !tandem && !tri) return 2;
    const int D = (int)Dd;
    const double L = D * LpD;
    if (basic) {
        // Generate_Cylinder: centre (Nx/5, Ny/2), cells i, j in 1..N, k in 0..Nz
        const double cx = Nx / 5.0, cy = Ny / 2.0;
        for (int i = 1; i <= Nx; i++)
            for (int j = 1; j <= Ny; j++)
                for (int k = 0; k <= Nz; k++)
                    if (std::sqrt(std::pow(cx - (i - 0.5), 2.0) + std::pow(cy - (j - 0.5), 2.0)) <= Dd / 2.0)
                        lb.fluid[i][j][k].type = TYPE_S;
        for (int i = 0; i <= Nx + 1; i++)
            for (int j = 0; j <= Ny + 1; j++)
                for (int k = 0; k <= Nz + 1; k++) {
                    LATTICE &c = lb.fluid[i][j][k];
                    if (i == 0) c.type = TYPE_IN;
                    if (i == Nx + 1) c.type = TYPE_OUT;
                    if (j == 0 || j == Ny + 1) c.type = TYPE_OUT;
                    if (c.type != TYPE_S) {
                        c.density = 1.0;
                        c.ux = u_max;
                    }
                }
        boxes.push_back({(int)(cx - Dd), (int)(cx + Dd), (int)(cy - Dd), (int)(cy + Dd)});
        g_lbm_options.ref_area = Dd;
    } else if (tandem) {
        // Generate_Circle for each circle: radius D/2 in integer division
        const int cx = Nx / 5;
        const int cy0 = (int)(Ny / 2 + L / 2);
        for (int n = 0; n < NB; n++) {
            const int cy = (int)(cy0 - n * L);
            for (int i = cx - D; i <= cx + D; i++)
                for (int j = cy - D; j <= cy + D; j++)
                    for (int k = 0; k <= Nz; k++)
                        if (std::sqrt(std::pow(cx - (i - 0.5), 2.0) + std::pow(cy - (j - 0.5), 2.0)) <= D / 2)
                            lb.fluid[i][j][k].type = TYPE_S;
            boxes.push_back({(int)(cx - L / 2), (int)(cx + L / 2), (int)(cy0 - n * L - L / 2), (int)(cy0 - n * L + L / 2)});
        }
        for (int i = 0; i <= Nx + 1; i++)
            for (int j = 0; j <= Ny + 1; j++)
                for (int k = 0; k <= Nz + 1; k++) {
                    LATTICE &c = lb.fluid[i][j][k];
                    if (j == 0 || j == Ny + 1) c.type = TYPE_OUT;
                    if (i == 0) c.type = TYPE_IN;
                    if (i == Nx + 1) c.type = TYPE_OUT;
                    if (c.type != TYPE_S) {
                        c.density = 1.0;
                        c.ux = u_max;
                    }
                }
        g_lbm_options.ref_area = D;
    } else {
        // Generate_Triangle: tip (Nx/5 + n L, Ny/2)
        const int tx = Nx / 5, ty = Ny / 2;
        for (int n = 0; n < NB; n++) {
            const int tip = (int)(tx + n * L);
            for (int i = 0; i <= D; i++)
                for (int j = (int)std::floor(-i / std::sqrt(3)); j <= (int)std::ceil(i / std::sqrt(3)); j++)
                    for (int k = 0; k <= Nz + 1; k++) lb.fluid[tip + i][ty + j][k].type = TYPE_S;
            boxes.push_back({(int)(tx + n * L - D / 4), (int)(tx + n * L + (D + L) / 2), ty - D, ty + D});
        }
        for (int i = 0; i <= Nx + 1; i++)
            for (int j = 0; j <= Ny + 1; j++)
                for (int k = 0; k <= Nz + 1; k++) {
                    LATTICE &c = lb.fluid[i][j][k];
                    if (j == 0 || j == Ny + 1) c.type = TYPE_OUT;
                    if (i == 0) c.type = TYPE_IN;
                    if (i == Nx + 1) c.type = TYPE_OUT;
                    if (k == 0 || k == Nz + 1) c.type = TYPE_F;
                    c.density = 1.0;
                    c.ux = c.type == TYPE_S ? 0.0 : u_max;
                }
        g_lbm_options.ref_area = 2.0 * D / std::sqrt(3.0);
    }
    lb.Init();
    const int nb = (int)boxes.size();
    std::vector<std::vector<double>> CL(nb), CD(nb);
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
        for (int n = 0; n < nb; n++) {
            const auto &b = boxes[n];
            CL[n].push_back(MEA_CL(lb, b[0], b[1], b[2], b[3], 1, 1));
            CD[n].push_back(MEA_CD(lb, b[0], b[1], b[2], b[3], 1, 1));
        }
    }
    FILE *fp = fopen(argv[10], "wb");
    if (!fp) return 3;
    for (int n = 0; n < nb; n++) fwrite(CL[n].data(), sizeof(double), CL[n].size(), fp);
    for (int n = 0; n < nb; n++) fwrite(CD[n].data(), sizeof(double), CD[n].size(), fp);
    fclose(fp);
    printf("{\"steps\": %lld, \"bodies\": %d}\n", lb.steps(), nb);
    return 0;
}
