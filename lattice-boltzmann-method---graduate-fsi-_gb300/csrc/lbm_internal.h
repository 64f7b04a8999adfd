// lbm_internal.h -- launcher interface between the C-ABI layer (lbm_abi.cu)
// and the kernel translation units.  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>

#include "lbm_device.cuh"

namespace lbmk {

// Launch plan of the staged (bulk-copy) step kernel; enabled = 0 falls back
// to the direct-load kernel.
struct TmaPlan {
    int enabled = 0;
    int ty = 0, grid = 0, per_sm = 0;  // rows per tile, CTAs, CTAs per SM
    long long ntiles = 0;
    size_t smem = 0;
};

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
    int thermal;
    int tx, ty;
    TmaPlan tma;
    cudaStream_t stream;
};

cudaError_t launch_step(int storage, const LaunchArgs &a);
cudaError_t plan_tma(int storage, bool thermal, const StepParams &P, int ty_pref, TmaPlan &tp);
cudaError_t launch_band_collide(int storage, const LaunchArgs &a, float fsign);
cudaError_t launch_init(int storage, void *A, void *GA, long long N, long long S, const float *fields,
                        const float init[5], bool thermal, cudaStream_t s);

// Immersed-boundary marker set on the device.
struct MarkerDev {
    int n;
    double *pos;     // [3][n] positions, reference node coordinates (node i at x = i)
    double *ds;      // [n] area (3D) weights
    float *udes;     // [3][n] desired velocity
    float *rho;      // [n] marker density
    float *force;    // [4][n] current F_m (x, y, z) and heat source Q_m
    double *acc;     // [4][n] sum over iterations of -F_m ds and Q_m ds (FP64)
    float *u0;       // [3][n] unforced interpolated velocity (assembled path)
    float *t0;       // [n] unforced interpolated temperature (assembled path)
    float tdes;      // desired marker temperature (thermal IBM)
};

struct IbmArgs {
    const StepParams *P;
    MarkerDev mk;
    DevState *ds;
    float *band;
    int thermal;
    cudaStream_t stream;
};

// first = 1: unforced interpolation and marker density; each call computes
// the interpolated velocity (and temperature) and the next marker force.
cudaError_t launch_ibm_interp(const IbmArgs &a, int first);
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
};
cudaError_t launch_ibm_finish(const IbmArgs &a, const BodyParams &bp, double *hist, long long hist_cap);

// Assembled IBM phase (marker-space iteration, see lbm_ibm.cu).
struct AsmPlan {
    int enabled = 0;
    int *pair_ptr = nullptr, *pair_idx = nullptr;  // marker neighbour lists (CSR)
    float *pairA = nullptr, *pairB = nullptr;      // coupling values, assembled each step
    int *node_ptr = nullptr, *node_mk = nullptr;   // band node -> covering markers (fixed body)
};
cudaError_t lbmk_iterate_smem(int n_markers);  // opt the one-CTA iteration into its shared memory
cudaError_t launch_ibm_assembled(int storage, bool lattice_thermal, const IbmArgs &a, const AsmPlan &ap, void *B,
                                 void *GB, float fsign, int m_max, double *hist, long long hist_cap,
                                 const BodyParams &bp, const LaunchArgs &la);

}  // namespace lbmk
