// dropin_details.cpp -- the reference's time loop in MORE_DETAILS mode
// (main.cpp:212-223 and 389: Sup_MacroProp at the output cadence) on the
// lid-driven cavity, through the LBM.h facade built with -DMORE_DETAILS.
// usage: dropin_details N STEPS OUT.bin
// Writes, for the interior cells (x fastest), as doubles: pressure,
// sigma[3][3], avg_velocity[3], avg_pressure, avg_ReynoldStress[3][3],
// rms_velocity[3], rms_pressure, rms_ReynoldStress[3][3]; and the
// OutputAVGVTK file ./avgfield.vtr of the last state.
#include <cstdio>
#include <cstdlib>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s N STEPS OUT.bin\n", argv[0]);
        return 2;
    }
    const int n = atoi(argv[1]), steps = atoi(argv[2]);
    const double tau = 0.8, lid = 0.05;
    g_lbm_options.u_max = 0.1;
    LBM lb(n, n, n, tau);
    for (int i = 0; i <= n + 1; i++)
        for (int j = 0; j <= n + 1; j++)
            for (int k = 0; k <= n + 1; k++) {
                bool ghost = i == 0 || i == n + 1 || j == 0 || j == n + 1 || k == 0 || k == n + 1;
                lb.fluid[i][j][k].type = ghost ? TYPE_S : TYPE_F;
                if (j == n + 1) lb.fluid[i][j][k].ux = lid;
            }
    lb.Init();
    int nout = 0;
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
        if (step % g_lbm_options.Nt == 0) {
            nout++;
            lb.Sup_MacroProp(step);
        }
    }
    OutputAVGVTK(nout, lb);
    lb.sync_to_host();
    FILE *fp = fopen(argv[3], "wb");
    if (!fp) return 3;
    for (int q = 0; q < 36; q++)
        for (int k = 1; k <= n; k++)
            for (int j = 1; j <= n; j++)
                for (int i = 1; i <= n; i++) {
                    const LATTICE &c = lb.fluid[i][j][k];
                    double v = 0;
                    if (q == 0) v = c.pressure;
                    else if (q < 10) v = c.sigma[(q - 1) / 3][(q - 1) % 3];
                    else if (q < 13) v = c.avg_velocity[q - 10];
                    else if (q == 13) v = c.avg_pressure;
                    else if (q < 23) v = c.avg_ReynoldStress[(q - 14) / 3][(q - 14) % 3];
                    else if (q < 26) v = c.rms_velocity[q - 23];
                    else if (q == 26) v = c.rms_pressure;
                    else v = c.rms_ReynoldStress[(q - 27) / 3][(q - 27) % 3];
                    fwrite(&v, sizeof(double), 1, fp);
                }
    fclose(fp);
    printf("{\"steps\": %lld}\n", lb.steps());
    return 0;
}
