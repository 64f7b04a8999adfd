// dropin_cylinder2d.cpp -- the reference's shipped default build
// (#define D2Q9, Cylinder_IBM, implicit forcing) through the LBM.h facade
// built with -DD2Q9: main_setup_Cylinder_IBM (lbm.cpp:1828-1854),
// Generate_Cylinder_Marker (lbm.cpp:1857-1877), the arc-length weights of
// main.cpp:123-131 and the IBM loop of main.cpp:195-205, with the reference's
// literal IBLBM options.  "transverse A F" runs its
// Cylinder_Transverse_Oscillation variant instead (u = 0.05, Re = 100,
// markers at center_y + A, V_solid = pi D^2 / 4 (Nz + 2)).  "vtk Nt" adds the
// main loop's output calls (main.cpp:62-66, 205-237): OutputVTK and
// OutputVTK_Marker of the initial state and every Nt steps, and OutputCSV of
// Cl and Cd under the reference's file names at each output (the reference
// rewrites the same two files after every step), into the working directory.
// usage: dropin_cylinder2d NX NY D NODES M_MAX STEPS OUT.csv [storage [transverse A F] [vtk Nt]]
// Writes step, Cd, Cl per step.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "LBM.h"

int main(int argc, char **argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: %s NX NY D NODES M_MAX STEPS OUT.csv [storage [transverse A F] [vtk Nt]]\n",
                argv[0]);
        return 2;
    }
    const int Nx = atoi(argv[1]), Ny = atoi(argv[2]), Nz = 1;
    const double D = atof(argv[3]);
    const int nodes = atoi(argv[4]), steps = atoi(argv[6]);
    lbm_options &o = g_lbm_options;
    o.m_max = atoi(argv[5]);
    if (argc > 8) o.storage = atoi(argv[8]);
    bool transverse = false;
    double amplitude = 0.0, frequency = 0.0;
    int Nt = 0;
    for (int a = 9; a < argc; a++) {
        if (strcmp(argv[a], "transverse") == 0 && a + 2 < argc) {
            transverse = true;
            amplitude = atof(argv[a + 1]);
            frequency = atof(argv[a + 2]);
            a += 2;
        } else if (strcmp(argv[a], "vtk") == 0 && a + 1 < argc) {
            Nt = atoi(argv[a + 1]);
            a += 1;
        }
    }
    const double u_max = transverse ? 0.05 : 0.1, Re = transverse ? 100.0 : 40.0;
    const double nu = u_max * D / Re, tau = 0.5 + nu / (1.0 / 3.0);
    const double center_x = Nx / 5.0, center_y = Ny / 2.0;
    // the reference's literal IBLBM (lbm.cpp:1259-1416)
    o.u_max = u_max;
    if (Nt > 0) o.Nt = Nt;
    o.csv_time_step = u_max / D;  // OutputCSV's (i + 1) dt u_max / D of the IBM cylinders
    o.ref_area = D;
    o.body_radius = D / 2;
    o.literal_sign = 1;
    o.rho_nearest = 1;
    o.added_mass = 1;
    o.vsolid = PI * D * D * 0.25 * (transverse ? (Nz + 2) : 1);
    o.body_center_set = 1;
    o.body_center[0] = center_x;
    o.body_center[1] = center_y;
    o.body_center[2] = 1;
    if (transverse) {
        o.motion = LBM_MOTION_TRANSVERSE_OSC;
        o.motion_amp = amplitude;
        o.motion_freq = frequency;
    }
    LBM lb(Nx, Ny, Nz, tau);
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int k = 0; k <= Nz + 1; k++) {
                LATTICE &c = lb.fluid[i][j][k];
                if (i == 0) c.type = TYPE_IN;
                if (i == Nx + 1) c.type = TYPE_OUT;
                if (j == 0 || j == Ny + 1) c.type = TYPE_OUT;
                c.density = 1.0;
                c.ux = u_max;
            }
    std::vector<MARKER> marker(nodes);
    const double radius = D / 2.0;
    for (int i = 0; i < nodes; i++) {
        marker[i].x = radius * cos(2 * PI / nodes * i) + center_x + 0.5;
        marker[i].y = radius * sin(2 * PI / nodes * i) + center_y + amplitude + 0.5;
        marker[i].z = 1;
    }
    for (int n = 0; n < nodes; n++) {
        const int n2 = (n + 1) % nodes;
        marker[n].Normal_Marker(n, marker[n].x, marker[n2].x, marker[n].y, marker[n2].y, marker[n].z, marker[n2].z);
    }
    std::vector<double> ds;
    for (int i = 0; i < nodes; i++) {
        const int j = (i + 1) % nodes;
        const double dx_ = marker[i].x - marker[j].x, dy_ = marker[i].y - marker[j].y, dz_ = marker[i].z - marker[j].z;
        ds.push_back(sqrt(pow(dx_, 2) + pow(dy_, 2) + pow(dz_, 2)));
    }
    lb.Init();
    int step = 0, n = 0;
    if (Nt > 0) {
        OutputVTK(step, lb);
        OutputVTK_Marker(step, marker);
    }
    std::vector<double> CL, CD;
    double V_CM[3] = {0, 0, 0};
    char name[96];
    for (step = 1; step <= steps; step++) {
        IBLBM(lb, marker, ds, CL, CD, V_CM, step * 1.0);
        lb.Collision();
        lb.Streaming();
        if (Nt > 0 && step % Nt == 0) {
            n++;
            OutputVTK(n, lb);
            OutputVTK_Marker(step, marker);
            snprintf(name, sizeof(name), "Cl at Re = %f.csv", Re);
            OutputCSV(CL, name);
            snprintf(name, sizeof(name), "Cd at Re = %f.csv", Re);
            OutputCSV(CD, name);
        }
    }
    FILE *fp = fopen(argv[7], "w");
    if (!fp) return 3;
    fprintf(fp, "step,cd,cl\n");
    for (size_t s = 0; s < CD.size(); s++) fprintf(fp, "%zu,%.17g,%.17g\n", s + 1, CD[s], CL[s]);
    fclose(fp);
    printf("{\"steps\": %lld, \"cd\": %.8g}\n", lb.steps(), CD.empty() ? 0.0 : CD.back());
    return 0;
}
