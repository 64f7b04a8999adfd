// dropin_cavity.cpp -- the reference's non-IBM time loop (main.cpp:212-221)
// on the lid-driven cavity, unchanged except for the set-up, through the
// LBM.h facade.  usage: dropin_cavity N STEPS OUT.bin [storage 0|1|2]
// Writes rho, ux, uy, uz of the interior cells (x fastest) as doubles.
#include <cstdio>
#include <cstdlib>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 4) {
        fprintf(stderr, "usage: %s N STEPS OUT.bin [storage]\n", argv[0]);
        return 2;
    }
    const int n = atoi(argv[1]), steps = atoi(argv[2]);
    if (argc > 4) g_lbm_options.storage = atoi(argv[4]);
    const double tau = 0.8, lid = 0.05;
    LBM lb(n, n, n, tau);
    for (int i = 0; i <= n + 1; i++)
        for (int j = 0; j <= n + 1; j++)
            for (int k = 0; k <= n + 1; k++) {
                bool ghost = i == 0 || i == n + 1 || j == 0 || j == n + 1 || k == 0 || k == n + 1;
                lb.fluid[i][j][k].type = ghost ? TYPE_S : TYPE_F;
                if (j == n + 1) lb.fluid[i][j][k].ux = lid;
            }
    lb.Init();
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
    }
    lb.sync_to_host();
    FILE *fp = fopen(argv[3], "wb");
    if (!fp) return 3;
    for (int q = 0; q < 4; q++)
        for (int k = 1; k <= n; k++)
            for (int j = 1; j <= n; j++)
                for (int i = 1; i <= n; i++) {
                    const LATTICE &c = lb.fluid[i][j][k];
                    double v = q == 0 ? c.density : q == 1 ? c.ux : q == 2 ? c.uy : c.uz;
                    fwrite(&v, sizeof(double), 1, fp);
                }
    fclose(fp);
    printf("{\"steps\": %lld}\n", lb.steps());
    return 0;
}
