// lbm_handle.h -- the state behind an lbm_handle (C ABI in lbm_abi.cu; the
// asynchronous output in lbm_output.cu reads it too).  Not part of the
// public ABI.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_device.cuh"
#include "lbm_internal.h"

struct lbm_output;  // asynchronous writer (lbm_output.cu)
struct lbm2d;       // D2Q9 solve (lbm2d.cu)

using lbmk::BodyParams;
using lbmk::MarkerDev;
using lbmk::StepParams;
using lbmk::DevState;

struct lbm_handle {
    lbm_output *out = nullptr;            // asynchronous VTK writer, created on first use
    lbm_config cfg;
    StepParams P;
    cudaStream_t s = nullptr;
    size_t esize = 4;
    void *f[2] = {nullptr, nullptr};   // population buffers A/B (past the guard)
    void *g[2] = {nullptr, nullptr};
    void *fraw[2] = {nullptr, nullptr}; // allocations
    void *graw[2] = {nullptr, nullptr};
    int cur = 0;
    float *mom = nullptr;
    float *band = nullptr;
    double *nu_scratch = nullptr;  // lbmgpu_nusselt: per-block partials, counts and result, on first use
    DevState *ds = nullptr;
    bool inited = false;
    long long steps = 0;
    // IBM
    bool ibm = false;
    lbm_ibm_config icfg;
    MarkerDev mk;
    BodyParams bp;
    double *hist = nullptr;
    long long hist_cap = 1 << 16;
    // lbmgpu_get_forces: pinned, device-mapped rows of the ring and their
    // count, written by a kernel (grown on demand)
    double *fstage = nullptr;
    long long fstage_rows = 0;
    // graphs
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gsteps = 16;
    int tx = 128, ty = 2;
    int vcells = 0;                       // x-cells per thread of gather steps (k_stepv), 0 = k_step
    // interior solid cells and their momentum exchange
    bool solids = false;
    uint32_t *solid_d = nullptr, *near_d = nullptr;
    float *mea_part = nullptr;
    int *mea_blocks = nullptr;
    int n_mea_blocks = 0;
    double *mea_ring = nullptr;
    long long mea_cap = 1 << 16;
    int tile_x = 1, tile_y = 1;           // near-box rounding in x and y
    size_t dev_bytes = 0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaEvent_t> evpool;
    cudaStream_t s2 = nullptr;            // IBM stream (overlaps the far-region streaming)
    cudaStream_t s3 = nullptr;            // force reduction, beside the last spreading and band collision
    cudaEvent_t ev_near = nullptr, ev_ibm = nullptr, ev_acc = nullptr, ev_fin = nullptr;
    // asynchronous moment read-back (lbmgpu_download_all_f32_async): its own
    // copy stream, ordered after the export pass
    cudaStream_t s_dl = nullptr;
    cudaEvent_t ev_dl_exported = nullptr, ev_dl_copied = nullptr;
    bool dl_issued = false;
    // MORE_DETAILS mode (lbm_details.cu)
    bool details = false;
    float *det = nullptr;                 // [7][N]: p, sigma xx xy xz yy yz zz
    double *stats = nullptr;              // [20][N]: Sup_MacroProp averages and rms values
    int stat_samples = 0;                 // samples folded in
    double stat_told = 0.0;               // told of the latest sample
    // D2Q9 handles (lattice = 9): everything lives in d2; the fields above
    // other than cfg, s, ev, esize, steps, inited and dev_bytes stay unused
    lbm2d *d2 = nullptr;
};

// D2Q9 solves (lbm2d.cu), reached through the same entry points.
lbm_status l2d_create(lbm_handle *h);
void l2d_free(lbm_handle *h);
lbm_status l2d_init(lbm_handle *h, const double *rho, const double *ux, const double *uy);
lbm_status l2d_set_markers(lbm_handle *h, const lbm_ibm_config *ic, const double *xyz, const double *ds);
lbm_status l2d_set_normals(lbm_handle *h, const double *nxyz);
lbm_status l2d_step(lbm_handle *h, int nsteps);
lbm_status l2d_download_f32(lbm_handle *h, int field, float *host);
lbm_status l2d_download_all_f32(lbm_handle *h, float *host);
lbm_status l2d_get_forces(lbm_handle *h, double *out, int max_steps, int *n_out);
lbm_status l2d_get_markers(lbm_handle *h, double *xyz);
lbm_status l2d_get_body(lbm_handle *h, double out[9]);
lbm_status l2d_status(lbm_handle *h, uint32_t *flags);
lbm_status l2d_set_solids(lbm_handle *h, const uint8_t *mask);
// after an export pass: u_y and T of the current moments, the solid-cell masks, the cell count
lbm_status l2d_thermal_moments(lbm_handle *h, const float **uy, const float **T, const uint16_t **links, long long *N);
lbm_status l2d_mea_box(lbm_handle *h, const int box[6], double out[3]);
// For the VTK writer: the current moments in the 3D layout ([8][N] when ENERGY,
// else [4][N]), and with an IBM body the force the box cells collided with
// ([2][nb], box order) and the box {x0, y0, width, height} of that pass.
lbm_status l2d_vtk_snapshot(lbm_handle *h, float *host, std::vector<float> &boxF, int box[4]);
// Checkpoint of a D2Q9 handle: the device regions the next step reads (the
// populations of buffer `src`, the current one when src < 0), a description
// of the configuration for the
// header, and the host-side state set after the regions were written back.
struct l2d_region {
    void *dev;
    size_t bytes;
    int both;  // 1: the populations, written into both buffers on restore
};
std::vector<l2d_region> l2d_checkpoint_regions(lbm_handle *h, int src);
// MORE_DETAILS of a D2Q9 handle into h->det / h->stats (cells: l2d_cells).
long long l2d_cells(lbm_handle *h);
float *l2d_moments(lbm_handle *h);  // the export's rows rho, ux, uy [, T, qx, qy]
cudaError_t l2d_details_async(lbm_handle *h, int fold, double told, double dt);
bool l2d_has_markers(lbm_handle *h);
void l2d_checkpoint_shape(lbm_handle *h, int shape[8]);
lbm_status l2d_checkpoint_restored(lbm_handle *h, long long steps);
int l2d_marker_count(lbm_handle *h);

// Launch the gather-only export of the current state's moments into h->mom
// (rho, ux, uy, uz [, T]) on h->s.
cudaError_t lbm_export_moments_async(lbm_handle *h);
void lbm_set_last_error(const std::string &m);
// Order h->s after the asynchronous output's read of h->mom (no-op without one).
cudaError_t lbm_mom_acquire(lbm_handle *h);
void lbm_output_free(lbm_handle *h);
// The moment export followed by the MORE_DETAILS pass into h->det on h->s;
// fold = 1 also folds the state into h->stats with Sup_MacroProp's told, dt.
cudaError_t lbm_details_async(lbm_handle *h, int fold, double told, double dt);
