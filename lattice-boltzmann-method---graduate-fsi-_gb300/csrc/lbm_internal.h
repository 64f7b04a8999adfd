// lbm_internal.h -- launcher interface between the C-ABI layer (lbm_abi.cu)
// and the kernel translation units.  Not part of the public ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "lbm_device.cuh"

namespace lbmk {

struct LaunchArgs {
    const StepParams *P;
    const void *A;
    void *B;
    const void *GA;
    void *GB;
    DevState *ds;
    float *mom;
    float *band;
    int gather;
    int export_only;
    int region;  // 0 all cells, 1 all but the IBM near box, 2 the near box only
    int thermal;
    int tx, ty;
    cudaStream_t stream;
    int pdl = 0;           // band collision: programmatic dependent launch behind the IBM chain
    int vcells = 0;        // > 1: gather steps use k_stepv with this many x-cells per thread
};

cudaError_t launch_step(int storage, const LaunchArgs &a);
// k_stepv (lbm_stepv.cu): whether it can run this lattice with vcells cells
// per thread, and its launcher.
bool step_vec_usable(int storage, const StepParams &P, int vcells);
cudaError_t launch_step_vec(int storage, const LaunchArgs &a);
cudaError_t launch_band_collide(int storage, const LaunchArgs &a, float fsign);
// Initial populations (equilibrium of the given or uniform fields) into A,
// GA and, when non-null, also into A2 / GA2.
cudaError_t launch_init(int storage, void *A, void *GA, void *A2, void *GA2, long long N, long long S,
                        const float *fields, const float init[5], bool thermal, cudaStream_t s);
// Momentum-exchange record of one step: fixed-order FP64 sum of the listed
// per-block partials into the ring (Fx, Fy, Fz, step) -- the force on the
// solid cells, minus the sums.
cudaError_t launch_mea_finish(const float *part, const int *blocks, int nblocks, double *ring, long long ring_cap,
                              DevState *ds, int advance, cudaStream_t s);

// Blocks of the free body's internal-fluid momentum sum (k_body_internal).
constexpr int kBodyBlocks = 64;

// Immersed-boundary marker set on the device.
struct MarkerDev {
    int n;
    double *pos;     // [3][n] positions, reference node coordinates (node i at x = i)
    double *ds;      // [n] area (3D) weights
    float *udes;     // [3][n] desired velocity
    float *rho;      // [n] marker density
    float *force;    // [4][n] current F_m (x, y, z) and heat source Q_m
    double *acc;     // [11][n] FP64: rows 0-3 the running sums over the iterations of -F_m ds and
                     // Q_m ds; rows 4-10 the step's force, torque about the body centre and heat
                     // of each marker, written by the last interpolation
    int *sb;         // [3][n] stencil origin of the step, band coordinates
    float *sw;       // [12][n] the step's Peskin weights per axis: x (4), y (4), z (4)
    double *ipart;   // [kBodyBlocks][6] free body: per-block FP64 partials of the internal-fluid momentum
    float tdes;      // desired marker temperature (thermal IBM)
};

struct IbmArgs {
    const StepParams *P;
    MarkerDev mk;
    DevState *ds;
    float *band;
    int thermal;
    cudaStream_t stream;
    int pdl = 0;  // programmatic dependent launch for the chain (FP32 storage, where the chain is the critical path)
};

// first = 1: unforced interpolation and marker density; each call computes
// the interpolated velocity (and temperature) and the next marker force.
cudaError_t launch_ibm_interp(const IbmArgs &a, int first, int last);
cudaError_t launch_ibm_spread(const IbmArgs &a);

// FP64 force/torque/heat reduction, history append and (optionally) the
// Newton-Euler rigid-body update that moves the markers and the band.
struct BodyParams {
    int free_body;
    double radius;
    double mass;       // rho_s V_s (rho_f = 1)
    double inertia;    // I_p
    double gacc[3];    // (1 - rho_f / rho_s) g
    int dof;           // bits 0-2 translation, 3-5 rotation
    double vol;        // V_s
    double grav[3];    // g
    double mv, iv;     // virtual mass C_v rho_f V_s and moment of inertia C_v 2/5 rho_f V_s R^2
};
cudaError_t launch_ibm_finish(const IbmArgs &a, const BodyParams &bp, double *hist, long long hist_cap);

}  // namespace lbmk
