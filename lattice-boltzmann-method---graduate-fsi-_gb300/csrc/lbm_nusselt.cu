// lbm_nusselt.cu -- Find_Nusselt_number (lbm.cpp:3538-3561) on the device:
// Nu = 1 + <u_y T> / (alpha dT / (Ny + 1)), <.> the mean over the fluid
// cells of the current MacroProp moments.  Every block sums its cells in a
// fixed order and a single thread adds the block sums in order, so the
// result does not depend on scheduling (the reference's OpenMP sum races).
#include <cuda_runtime.h>

#include <string>

#include "lbm_handle.h"

namespace {

constexpr int kNuBlocks = 304;  // two per SM
constexpr int kNuThreads = 256;

__global__ void __launch_bounds__(kNuThreads) k_nusselt_part(const float *__restrict__ uy, const float *__restrict__ T,
                                                             long long N, const uint32_t *__restrict__ solid3,
                                                             const uint16_t *__restrict__ links2,
                                                             double *__restrict__ part,
                                                             unsigned long long *__restrict__ cnt) {
    __shared__ double ss[kNuThreads];
    __shared__ unsigned long long sc[kNuThreads];
    double s = 0.0;
    unsigned long long n = 0;
    for (long long c = blockIdx.x * (long long)kNuThreads + threadIdx.x; c < N; c += (long long)kNuBlocks * kNuThreads) {
        bool solid = false;
        if (solid3) solid = (solid3[c >> 5] >> (c & 31)) & 1u;
        if (links2) solid = (links2[c] & 0x8000u) != 0;
        if (solid) continue;
        s += (double)uy[c] * (double)T[c];
        n++;
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = n;
    __syncthreads();
    for (int h = kNuThreads / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) {
            ss[threadIdx.x] += ss[threadIdx.x + h];
            sc[threadIdx.x] += sc[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = ss[0];
        cnt[blockIdx.x] = sc[0];
    }
}

__global__ void k_nusselt_finish(const double *__restrict__ part, const unsigned long long *__restrict__ cnt,
                                 double *__restrict__ out) {
    double s = 0.0;
    unsigned long long n = 0;
    for (int b = 0; b < kNuBlocks; b++) {
        s += part[b];
        n += cnt[b];
    }
    out[0] = s;
    out[1] = (double)n;
}

lbm_status fail_nu(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

}  // namespace

extern "C" lbm_status lbmgpu_nusselt(lbm_handle *h, double alpha, double dT, double *out) {
    if (!h || !out) return fail_nu(LBM_ERR_INVALID, "nusselt: null argument");
    if (!(alpha > 0) || dT == 0) return fail_nu(LBM_ERR_INVALID, "nusselt: alpha > 0 and dT != 0 needed");
    if (!h->inited) return fail_nu(LBM_ERR_STATE, "nusselt: call lbmgpu_init first");
    const float *uy = nullptr, *T = nullptr;
    const uint32_t *solid3 = nullptr;
    const uint16_t *links2 = nullptr;
    long long N = 0;
    int ny_dev = h->cfg.ny;
    if (h->d2) {
        lbm_status s = l2d_thermal_moments(h, &uy, &T, &links2, &N);
        if (s != LBM_OK) return s;
    } else {
        if (!h->cfg.thermal) return fail_nu(LBM_ERR_STATE, "nusselt: the handle has no temperature");
        cudaError_t e = lbm_export_moments_async(h);
        if (e != cudaSuccess) return fail_nu(LBM_ERR_CUDA, std::string("nusselt: ") + cudaGetErrorString(e));
        N = h->P.N;
        uy = h->mom + 2 * N;
        T = h->mom + 4 * N;
        solid3 = h->solid_d;
    }
    // the reference's Ny: a periodic y axis carries its two ghost rows on the device
    const int Ny = h->cfg.faces[2].kind == LBM_FACE_PERIODIC ? ny_dev - 2 : ny_dev;
    // partials, counts and the result: one allocation per handle, made on the
    // first call (a cudaFree on every call would synchronise the device)
    cudaError_t e = cudaSuccess;
    if (!h->nu_scratch) e = cudaMalloc((void **)&h->nu_scratch, (2 * kNuBlocks + 2) * sizeof(double));
    double *part = h->nu_scratch;
    unsigned long long *cnt = reinterpret_cast<unsigned long long *>(h->nu_scratch + kNuBlocks);
    double *res = h->nu_scratch + 2 * kNuBlocks;
    if (e == cudaSuccess) {
        k_nusselt_part<<<kNuBlocks, kNuThreads, 0, h->s>>>(uy, T, N, solid3, links2, part, cnt);
        k_nusselt_finish<<<1, 1, 0, h->s>>>(part, cnt, res);
        e = cudaGetLastError();
    }
    double r[2] = {0.0, 0.0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, res, sizeof(r), cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return fail_nu(LBM_ERR_CUDA, std::string("nusselt: ") + cudaGetErrorString(e));
    if (r[1] < 1) return fail_nu(LBM_ERR_STATE, "nusselt: no fluid cell");
    out[0] = 1.0 + (r[0] / r[1]) / (alpha * dT / (Ny + 1));
    return LBM_OK;
}
