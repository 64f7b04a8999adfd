// dropin_sphere.cpp -- the reference's IBM time loop (main.cpp:195-211:
// IBLBM -> Collision -> Streaming, Cl/Cd appended every step) on a channel
// with an immersed sphere, through the LBM.h facade.
// usage: dropin_sphere NX NY NZ TAU D NMARKERS STEPS OUT.csv [storage]
// Markers: Fibonacci sphere centred at (NX/4, NY/2, NZ/2), area weights
// pi D^2 / N.  Inlet TYPE_IN at i = 0 and TYPE_OUT elsewhere on the x faces
// (the reference's Sphere_BB/IBM set-up, lbm.cpp:1799-1818) with walls on y, z.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 9) {
        fprintf(stderr, "usage: %s NX NY NZ TAU D NMARKERS STEPS OUT.csv [storage]\n", argv[0]);
        return 2;
    }
    const int Nx = atoi(argv[1]), Ny = atoi(argv[2]), Nz = atoi(argv[3]);
    const double tau = atof(argv[4]), D = atof(argv[5]);
    const int nm = atoi(argv[6]), steps = atoi(argv[7]);
    if (argc > 9) g_lbm_options.storage = atoi(argv[9]);
    const double u_max = 0.05, PI = 3.14159265;
    g_lbm_options.u_max = u_max;
    g_lbm_options.ref_area = PI * D * D / 4;
    g_lbm_options.body_radius = D / 2;
    LBM lb(Nx, Ny, Nz, tau);
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int k = 0; k <= Nz + 1; k++) {
                LATTICE &c = lb.fluid[i][j][k];
                if (i == 0) c.type = TYPE_IN;
                if (i == Nx + 1) c.type = TYPE_OUT;
                if (j == 0 || j == Ny + 1 || k == 0 || k == Nz + 1) c.type = TYPE_S;
                if (c.type != TYPE_S) c.ux = u_max;
            }
    std::vector<MARKER> marker(nm);
    const double cxm = Nx / 4.0, cym = Ny / 2.0, czm = Nz / 2.0, R = D / 2, ga = PI * (3.0 - std::sqrt(5.0));
    std::vector<double> ds(nm, PI * D * D / nm);
    for (int m = 0; m < nm; m++) {
        double zz = 1.0 - (2.0 * m + 1.0) / nm, r = std::sqrt(1.0 - zz * zz), ph = ga * m;
        marker[m].x = cxm + R * r * std::cos(ph);
        marker[m].y = cym + R * r * std::sin(ph);
        marker[m].z = czm + R * zz;
        marker[m].normal[0] = r * std::cos(ph);
        marker[m].normal[1] = r * std::sin(ph);
        marker[m].normal[2] = zz;
    }
    lb.Init();
    std::vector<double> CL, CD;
    double V_CM[3] = {0, 0, 0};
    for (int step = 1; step <= steps; step++) {
        IBLBM(lb, marker, ds, CL, CD, V_CM, step * 1.0);
        lb.Collision();
        lb.Streaming();
    }
    FILE *fp = fopen(argv[8], "w");
    if (!fp) return 3;
    fprintf(fp, "step,cd,cl\n");
    for (size_t s = 0; s < CD.size(); s++) fprintf(fp, "%zu,%.17g,%.17g\n", s + 1, CD[s], CL[s]);
    fclose(fp);
    printf("{\"steps\": %lld, \"cd\": %.8g}\n", lb.steps(), CD.empty() ? 0.0 : CD.back());
    return 0;
}
