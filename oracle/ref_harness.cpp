// ref_harness.cpp -- driver for the reference-literal oracle build.
//
// Test infrastructure only.  It replaces main.cpp (which has a VTK/CSV output
// cadence and an interactive prompt) with a batch driver that
//   - builds the geometry through the reference's public LBM::fluid array
//     (the cavity) or the reference's own setup functions (the cylinder),
//   - runs the reference's own Init / Collision / Streaming / MacroProp and
//     IBLBM in the order of main.cpp:195-221,
//   - times only the step loop (wall clock), and
//   - dumps rho, u (and F, Cl, Cd for the IBM case; Cl, Cd of the
//     momentum exchange after every step for the staircase sphere; in
//     MORE_DETAILS mode the pressure, the viscous stress and the
//     Sup_MacroProp averages and rms values) as raw doubles, x fastest, ghost
//     layers included.
#include "LBM.h"

#include <omp.h>

#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <vector>

static void dump_field(LBM &lb, FILE *fp, int which) {
    int NX = Nx + 2, NY = Ny + 2, NZ = Nz + 2;
    std::vector<double> buf((size_t)NX * NY * NZ);
    for (int k = 0; k < NZ; k++)
        for (int j = 0; j < NY; j++)
            for (int i = 0; i < NX; i++) {
                LATTICE &c = lb.fluid[i][j][k];
                double v = 0;
                switch (which) {
                case 0: v = c.density; break;
                case 1: v = c.ux; break;
                case 2: v = c.uy; break;
                case 3: v = c.uz; break;
                case 4: v = c.F[0]; break;
                case 5: v = c.F[1]; break;
                case 6: v = c.F[2]; break;
#if defined ENERGY
                // 50: T; 51..53: heat flux q
                case 50: v = c.T; break;
                case 51: v = c.q[0]; break;
                case 52: v = c.q[1]; break;
                case 53: v = c.q[2]; break;
#endif
#if defined MORE_DETAILS
                // 7: pressure; 8..16: sigma[a][b]; 17..19: avg_velocity;
                // 20: avg_pressure; 21..29: avg_ReynoldStress; 30..32:
                // rms_velocity; 33: rms_pressure; 34..42: rms_ReynoldStress
                case 7: v = c.pressure; break;
                case 20: v = c.avg_pressure; break;
                case 33: v = c.rms_pressure; break;
                default:
                    if (which >= 8 && which <= 16) v = c.sigma[(which - 8) / 3][(which - 8) % 3];
                    if (which >= 17 && which <= 19) v = c.avg_velocity[which - 17];
                    if (which >= 21 && which <= 29) v = c.avg_ReynoldStress[(which - 21) / 3][(which - 21) % 3];
                    if (which >= 30 && which <= 32) v = c.rms_velocity[which - 30];
                    if (which >= 34 && which <= 42) v = c.rms_ReynoldStress[(which - 34) / 3][(which - 34) % 3];
                    break;
#endif
                }
                buf[(size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k)] = v;
            }
    fwrite(buf.data(), sizeof(double), buf.size(), fp);
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s steps out.bin [lid_velocity [vtk]]  (cylinders: steps out.bin [vtk])\n", argv[0]);
        return 2;
    }
    int steps = atoi(argv[1]);
    const char *out = argv[2];
#if defined REF_CAVITY
    double lid = argc > 3 ? atof(argv[3]) : 0.05;
    LBM lb(Nx, Ny, Nz, tau);
    for (int i = 0; i <= Nx + 1; i++)
        for (int j = 0; j <= Ny + 1; j++)
            for (int k = 0; k <= Nz + 1; k++) {
                bool ghost = i == 0 || i == Nx + 1 || j == 0 || j == Ny + 1 || k == 0 || k == Nz + 1;
                lb.fluid[i][j][k].type = ghost ? TYPE_S : TYPE_F;
                // moving lid: the whole ghost plane j = Ny+1 (Couette "top wall"
                // convention, lbm.cpp:1548-1551)
                if (j == Ny + 1) lb.fluid[i][j][k].ux = lid;
            }
    lb.Init();
    double t0 = omp_get_wtime();
    for (int s = 1; s <= steps; s++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
#if defined MORE_DETAILS
        // the call of main.cpp:389, made at the output cadence (main.cpp:223)
        if (s % Nt == 0) lb.Sup_MacroProp(s);
#endif
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 4; w++) dump_field(lb, fp, w);
#if defined MORE_DETAILS
    for (int w = 7; w <= 42; w++) dump_field(lb, fp, w);
#endif
    fclose(fp);
    if (argc > 4) {
        // the reference's own VTK writer (lbm.cpp:2290-2642): ./field000000.vtr
        int nout = 0;
        OutputVTK(nout, lb);
    }
    double mlups = (double)Nx * Ny * Nz * steps / (t1 - t0) / 1e6;
    printf("{\"case\": \"cavity\", \"nx\": %d, \"steps\": %d, \"seconds\": %.6f, \"mlups\": %.4f, \"threads\": %d}\n",
           Nx, steps, t1 - t0, mlups, omp_get_max_threads());
#elif defined REF_CYLINDER || defined REF_TRANSVERSE || defined REF_INLINE || defined REF_ARBIE
#if defined REF_TRANSVERSE
    LBM lb = main_setup_Cylinder_TransverseOscillating();
#elif defined REF_INLINE
    LBM lb = main_setup_Cylinder_InlineOscillating();
#elif defined REF_ARBIE
    LBM lb = main_setup_Cylinder_IBM_Moving();
#else
    LBM lb = main_setup_Cylinder_IBM();
#endif
    std::vector<MARKER> marker(number_nodes);
    Generate_Cylinder_Marker(marker);
    // arc-length weights as main.cpp:123-131 computes them
    std::vector<double> ds;
    for (int i = 0; i < number_nodes; i++) {
        int j = (i + 1) % number_nodes;
        double ddx = marker[i].x - marker[j].x, ddy = marker[i].y - marker[j].y, ddz = marker[i].z - marker[j].z;
        ds.push_back(sqrt(pow(ddx, 2) + pow(ddy, 2) + pow(ddz, 2)));
    }
    double V_CM[3] = {0, 0, 0};
    std::vector<double> CL, CD;
    lb.Init();
    double t0 = omp_get_wtime();
    for (int step = 1; step <= steps; step++) {
        IBLBM(lb, marker, ds, CL, CD, V_CM, step * dt);
        lb.Collision();
        lb.Streaming();
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 7; w++) dump_field(lb, fp, w);
    fwrite(CL.data(), sizeof(double), CL.size(), fp);
    fwrite(CD.data(), sizeof(double), CD.size(), fp);
    for (int n = 0; n < number_nodes; n++) {
        double v[8] = {marker[n].x, marker[n].y, marker[n].z, marker[n].normal[0], marker[n].normal[1],
                       marker[n].normal[2], ds[n], 0.0};
        fwrite(v, sizeof(double), 8, fp);
    }
    fclose(fp);
    if (argc > 3) {
        // the reference's own writers: OutputVTK (lbm.cpp:2290-2642), ./field000000.vtr, and
        // OutputVTK_Marker (lbm.cpp:3033-3077) of the final markers
        int nout = 0;
        OutputVTK(nout, lb);
        OutputVTK_Marker(steps, marker);
    }
    double mlups = (double)Nx * Ny * Nz * steps / (t1 - t0) / 1e6;
    printf("{\"case\": \"cylinder2d\", \"nx\": %d, \"steps\": %d, \"seconds\": %.6f, \"mlups\": %.4f, \"threads\": %d}\n",
           Nx, steps, t1 - t0, mlups, omp_get_max_threads());
#elif defined REF_POISEUILLE
    LBM lb = main_setup_Poiseuille();
    lb.Init();
    double t0 = omp_get_wtime();
    for (int s = 1; s <= steps; s++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 4; w++) dump_field(lb, fp, w);
#if defined ENERGY
    for (int w = 50; w <= 53; w++) dump_field(lb, fp, w);
#endif
    fclose(fp);
    printf("{\"case\": \"poiseuille\", \"ny\": %d, \"steps\": %d, \"seconds\": %.6f}\n", Ny, steps, t1 - t0);
#elif defined REF_COUETTE
    LBM lb = main_setup_Couette();
#if defined REF_NEUMANN
    // the top wall as a Neumann wall: type_Energy TYPE_Q with LBM.h's
    // j_dot_n (Determine_Twall_Neumann, lbm.cpp:983-1028)
    for (int i = 0; i <= Nx + 1; i++)
        for (int k = 0; k <= Nz + 1; k++) lb.fluid[i][Ny + 1][k].type_Energy = TYPE_Q;
#endif
    lb.Init();
    double t0 = omp_get_wtime();
    for (int s = 1; s <= steps; s++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 4; w++) dump_field(lb, fp, w);
    for (int w = 50; w <= 53; w++) dump_field(lb, fp, w);
    fclose(fp);
    printf("{\"case\": \"couette_energy\", \"ny\": %d, \"steps\": %d, \"seconds\": %.6f}\n", Ny, steps, t1 - t0);
#elif defined REF_RAYLEIGH
    LBM lb = main_setup_RayleighBenard1();
    lb.Init();
    double t0 = omp_get_wtime();
    for (int s = 1; s <= steps; s++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 7; w++) dump_field(lb, fp, w);
    for (int w = 50; w <= 53; w++) dump_field(lb, fp, w);
    fclose(fp);
    printf("{\"case\": \"rayleigh_benard\", \"nx\": %d, \"ny\": %d, \"nz\": %d, \"steps\": %d, \"seconds\": %.6f}\n",
           Nx, Ny, Nz, steps, t1 - t0);
#elif defined REF_CYLBASIC || defined REF_TANDEM || defined REF_TRIANGLE
    // the staircase 2D bodies with the momentum exchange of main.cpp:242-356,
    // taken after every step (the reference takes it every Nt steps)
#if defined REF_CYLBASIC
    LBM lb = main_setup_Cylinder();
    const int nb = 1;
#elif defined REF_TANDEM
    LBM lb = main_setup_Tandem_Circle();
    const int nb = N;
#else
    LBM lb = main_setup_Tandem_Triangle();
    const int nb = N;
#endif
    std::vector<std::vector<double>> CL(nb), CD(nb);
    lb.Init();
    double t0 = omp_get_wtime();
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
#if defined MORE_DETAILS
        // the call of main.cpp:389, made at the output cadence (main.cpp:223)
        if (step % Nt == 0) lb.Sup_MacroProp(step);
#endif
        for (int n = 0; n < nb; n++) {
#if defined REF_CYLBASIC
            CL[n].push_back(MEA_CL(lb, center_x - D, center_x + D, center_y - D, center_y + D, 1, 1));
            CD[n].push_back(MEA_CD(lb, center_x - D, center_x + D, center_y - D, center_y + D, 1, 1));
#elif defined REF_TANDEM
            CL[n].push_back(MEA_CL(lb, center_x - L / 2, center_x + L / 2, center_y - n * L - L / 2,
                                   center_y - n * L + L / 2, 1, 1));
            CD[n].push_back(MEA_CD(lb, center_x - L / 2, center_x + L / 2, center_y - n * L - L / 2,
                                   center_y - n * L + L / 2, 1, 1));
#else
            CL[n].push_back(MEA_CL(lb, tip_x + n * L - D / 4, tip_x + n * L + (D + L) / 2, tip_y - D, tip_y + D, 1, 1));
            CD[n].push_back(MEA_CD(lb, tip_x + n * L - D / 4, tip_x + n * L + (D + L) / 2, tip_y - D, tip_y + D, 1, 1));
#endif
        }
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 4; w++) dump_field(lb, fp, w);
    for (int n = 0; n < nb; n++) {
        fwrite(CL[n].data(), sizeof(double), CL[n].size(), fp);
        fwrite(CD[n].data(), sizeof(double), CD[n].size(), fp);
    }
#if defined MORE_DETAILS
    for (int w = 7; w <= 42; w++) dump_field(lb, fp, w);
#endif
    fclose(fp);
#if defined MORE_DETAILS && defined REF_TRIANGLE
    // the reference's own writers, into the folders it names for this case
    // (lbm.cpp:2299-2301, 2654-2658): Flowfield/field000000.vtr and
    // avgfield.vtr under "./output Tandem Triangle/LpD = .. Re = ..", which
    // must exist
    if (argc > 4) {
        char dir[128], sub[160];
        snprintf(dir, sizeof(dir), "./output Tandem Triangle/LpD = %.1f Re = %.0f", LpD, Re);
        snprintf(sub, sizeof(sub), "%s/Flowfield", dir);
        mkdir("./output Tandem Triangle", 0755);
        mkdir(dir, 0755);
        mkdir(sub, 0755);
        int nout = 0;
        OutputVTK(nout, lb);
        OutputAVGVTK(nout, lb);
    }
#endif
    // the solid cells of the set-up, layer k = 1 (x fastest)
    if (argc > 3) {
        FILE *fs = fopen(argv[3], "wb");
        if (!fs) return 3;
        for (int j = 0; j <= Ny + 1; j++)
            for (int i = 0; i <= Nx + 1; i++) {
                unsigned char t = (unsigned char)lb.fluid[i][j][1].type;
                fwrite(&t, 1, 1, fs);
            }
        fclose(fs);
    }
    double mlups = (double)Nx * Ny * steps / (t1 - t0) / 1e6;
    printf("{\"case\": \"staircase2d\", \"nx\": %d, \"bodies\": %d, \"steps\": %d, \"seconds\": %.6f, \"mlups\": %.4f}\n",
           Nx, nb, steps, t1 - t0, mlups);
#elif defined REF_SPHERE
    LBM lb = main_setup_Sphere();
    std::vector<double> CL, CD;
    lb.Init();
    double t0 = omp_get_wtime();
    for (int step = 1; step <= steps; step++) {
        lb.Collision();
        lb.Streaming();
        lb.MacroProp();
        // the calls of main.cpp:369-372, every step
        CL.push_back(MEA_CL(lb, center_x - D, center_x + D, center_y - D, center_y + D, center_z - D, center_z + D));
        CD.push_back(MEA_CD(lb, center_x - D, center_x + D, center_y - D, center_y + D, center_z - D, center_z + D));
    }
    double t1 = omp_get_wtime();
    FILE *fp = fopen(out, "wb");
    if (!fp) return 3;
    for (int w = 0; w < 4; w++) dump_field(lb, fp, w);
    fwrite(CL.data(), sizeof(double), CL.size(), fp);
    fwrite(CD.data(), sizeof(double), CD.size(), fp);
    fclose(fp);
    double mlups = (double)Nx * Ny * Nz * steps / (t1 - t0) / 1e6;
    printf("{\"case\": \"sphere_bb\", \"nx\": %d, \"steps\": %d, \"seconds\": %.6f, \"mlups\": %.4f, \"threads\": %d}\n",
           Nx, steps, t1 - t0, mlups, omp_get_max_threads());
#endif
    return 0;
}
