// lbm_details.cu -- the reference's MORE_DETAILS quantities (LBM.h:55) on the
// device:
//
//   pressure      p = rho / 3                                   lbm.cpp:683
//   stress        sigma_ab = -(tau - 1/2)/tau sum_l f_l (c_la - u_a)(c_lb - u_b)
//                                                               lbm.cpp:687-705
//   statistics    the running averages and rms values of LBM::Sup_MacroProp
//                                                               lbm.cpp:865-939
//
// of the current (post-streaming) state.  One pass over the interior pulls
// the 19 populations of a cell exactly as the fused step does (same boundary
// classes, same bounce-back on solid cells), takes rho and u from the moment
// export that precedes it on the stream, and forms the central second moment
// from the raw one,
//     sum f (c - u)(c - u)^T = Pi - u j^T - j u^T + rho u u^T,
// Pi = sum f c c^T, j = sum f c (the shifted storage f - w adds cs^2 delta to
// Pi and nothing to j).  With a sample to fold in, the same pass updates the
// FP64 statistics in place.
//
// Layouts, [component][interior cell]:
//   details (FP32, 7):  p, sigma xx, xy, xz, yy, yz, zz
//   statistics (FP64, 20):  avg u (3), avg p, avg Reynolds stress (6),
//                           rms u (3), rms p, rms Reynolds stress (6)
// The reference never computes the vorticity (its code is commented out,
// lbm.cpp:712-770): its averages and rms values stay zero and are not held.
#include <cuda_runtime.h>

#include <string>

#include "lbm_handle.h"
#include "lbm_internal.h"
#include "lbm_step.cuh"

namespace lbmk {

constexpr int kDetailFields = 7;
constexpr int kStatFields = 20;

struct StatSample {
    int fold;     // 1: fold this state into the statistics
    double told;  // (n - Nt) dt of Sup_MacroProp(n)
    double dt;
};

template <class T, bool SOLID>
__global__ void __launch_bounds__(256) k_details(const T *__restrict__ A, const __grid_constant__ StepParams P,
                                                 const float *__restrict__ mom, float *__restrict__ det,
                                                 double *__restrict__ st, float sfac, int gather, StatSample smp) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z;
    const bool valid = x < P.nx && y < P.ny;
    const long long cell = valid ? (long long)x + (long long)P.nx * ((long long)y + (long long)P.ny * z) : 0;
    const int raw = valid ? ((x == 0 ? 1 : 0) | (x == P.nx - 1 ? 2 : 0) | (y == 0 ? 4 : 0) | (y == P.ny - 1 ? 8 : 0) |
                             (z == 0 ? 16 : 0) | (z == P.nz - 1 ? 32 : 0))
                          : 0;
    float f[Q];
    if (SOLID) {
        float g[QT], mea[3];
        const bool sc = valid && mask_bit(P.solid, cell);
        gather_solid<T, false>(A, nullptr, f, g, x, y, z, cell, raw, valid, sc, gather, P, mea);
    } else {
        const int rawrow = P.xface ? (raw & ~3) : raw;
        const bool bwarp = __any_sync(0xffffffffu, rawrow != 0);
        gather_flow<T>(A, f, x, y, z, cell, raw, valid, bwarp, gather, P);
    }
    if (!valid) return;
    float jx = 0.0f, jy = 0.0f, jz = 0.0f;
    float pxx = 0.0f, pxy = 0.0f, pxz = 0.0f, pyy = 0.0f, pyz = 0.0f, pzz = 0.0f;
#pragma unroll
    for (int l = 1; l < Q; l++) {
        const float v = f[l];
        const float ex = (float)cx(l), ey = (float)cy(l), ez = (float)cz(l);
        jx += ex * v;
        jy += ey * v;
        jz += ez * v;
        pxx += ex * ex * v;
        pxy += ex * ey * v;
        pxz += ex * ez * v;
        pyy += ey * ey * v;
        pyz += ey * ez * v;
        pzz += ez * ez * v;
    }
    const long long N = P.N;
    const float rho = mom[cell], ux = mom[N + cell], uy = mom[2 * N + cell], uz = mom[3 * N + cell];
    const float cs2 = 1.0f / 3.0f;
    const float sxx = (pxx + cs2) - 2.0f * ux * jx + rho * ux * ux;
    const float syy = (pyy + cs2) - 2.0f * uy * jy + rho * uy * uy;
    const float szz = (pzz + cs2) - 2.0f * uz * jz + rho * uz * uz;
    const float sxy = pxy - ux * jy - jx * uy + rho * ux * uy;
    const float sxz = pxz - ux * jz - jx * uz + rho * ux * uz;
    const float syz = pyz - uy * jz - jy * uz + rho * uy * uz;
    det[cell] = rho / 3.0f;
    det[N + cell] = sfac * sxx;
    det[2 * N + cell] = sfac * sxy;
    det[3 * N + cell] = sfac * sxz;
    det[4 * N + cell] = sfac * syy;
    det[5 * N + cell] = sfac * syz;
    det[6 * N + cell] = sfac * szz;
    if (!smp.fold) return;

    // Sup_MacroProp, in the reference's order and with its weights
    const double told = smp.told, dt = smp.dt, w1 = told + 1.0;
    const double u[3] = {ux, uy, uz};
    const double p = (double)rho / 3.0;
    double au[3], d[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        au[a] = (st[a * N + cell] * told + u[a] * dt) / (told + dt);
        st[a * N + cell] = au[a];
        d[a] = u[a] - au[a];
    }
    const double ap = (st[3 * N + cell] * told + p) / w1;
    st[3 * N + cell] = ap;
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
    double ars[6];
#pragma unroll
    for (int s = 0; s < 6; s++) {
        ars[s] = (st[(4 + s) * N + cell] * told + d[ia[s]] * d[ib[s]]) / w1;
        st[(4 + s) * N + cell] = ars[s];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double r = st[(10 + a) * N + cell];
        st[(10 + a) * N + cell] = sqrt((r * r * told + d[a] * d[a]) / w1);
    }
    // the pressure rms squares the current pressure (lbm.cpp:913)
    const double dp = p - ap;
    st[13 * N + cell] = sqrt((p * p * told + dp * dp) / w1);
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const double r = st[(14 + s) * N + cell];
        const double e = u[ia[s]] * u[ib[s]] - ars[s];
        st[(14 + s) * N + cell] = sqrt((r * r * told + e * e) / w1);
    }
}

template <class T>
static cudaError_t launch_details_t(const void *A, const StepParams &P, const float *mom, float *det, double *st,
                                   float sfac, int gather, StatSample smp, cudaStream_t s) {
    const dim3 block(32, 8, 1);
    const dim3 grid((P.nx + 31) / 32, (P.ny + 7) / 8, P.nz);
    if (P.solid != nullptr)
        k_details<T, true><<<grid, block, 0, s>>>((const T *)A, P, mom, det, st, sfac, gather, smp);
    else
        k_details<T, false><<<grid, block, 0, s>>>((const T *)A, P, mom, det, st, sfac, gather, smp);
    return cudaGetLastError();
}

}  // namespace lbmk

using lbmk::kDetailFields;
using lbmk::kStatFields;

namespace {

lbm_status det_fail(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

// cells of the handle's lattice (D3Q19 interior or D2Q9 device grid)
long long det_cells(lbm_handle *h) { return h->d2 ? l2d_cells(h) : h->P.N; }

}  // namespace

// Export the moments, then the details (and fold a statistics sample when
// smp_fold) of the current state on h->s.
cudaError_t lbm_details_async(lbm_handle *h, int smp_fold, double told, double dt) {
    if (h->d2) return l2d_details_async(h, smp_fold, told, dt);
    cudaError_t e = lbm_export_moments_async(h);
    if (e != cudaSuccess) return e;
    StepParams P = h->P;
    P.mea = nullptr;  // no momentum-exchange record from this pass
    lbmk::StatSample smp{smp_fold, told, dt};
    const float sfac = (float)(-(h->cfg.tau - 0.5) / h->cfg.tau);
    const int gather = h->steps == 0 ? 0 : 1;
    const void *A = h->f[h->cur];
    switch (h->cfg.storage) {
    case LBM_STORE_F16:
        return lbmk::launch_details_t<__half>(A, P, h->mom, h->det, h->stats, sfac, gather, smp, h->s);
    case LBM_STORE_BF16:
        return lbmk::launch_details_t<__nv_bfloat16>(A, P, h->mom, h->det, h->stats, sfac, gather, smp, h->s);
    default:
        return lbmk::launch_details_t<float>(A, P, h->mom, h->det, h->stats, sfac, gather, smp, h->s);
    }
}

extern "C" lbm_status lbmgpu_set_more_details(lbm_handle *h, int on) {
    if (!h) return det_fail(LBM_ERR_INVALID, "set_more_details: null handle");
    if (h->d2 && l2d_has_markers(h))
        return det_fail(LBM_ERR_UNSUPPORTED, "set_more_details: not for D2Q9 IBM handles (the reference's IBM loop "
                                             "never calls MacroProp, which forms the details)");
    if (lbmgpu_sync(h) != LBM_OK) return LBM_ERR_CUDA;
    if (!on) {
        if (h->det) cudaFree(h->det);
        if (h->stats) cudaFree(h->stats);
        if (h->det) h->dev_bytes -= (size_t)kDetailFields * det_cells(h) * sizeof(float);
        if (h->stats) h->dev_bytes -= (size_t)kStatFields * det_cells(h) * sizeof(double);
        h->det = nullptr;
        h->stats = nullptr;
        h->details = false;
        return LBM_OK;
    }
    if (h->details) return LBM_OK;
    const size_t N = (size_t)det_cells(h);
    if (cudaMalloc((void **)&h->det, kDetailFields * N * sizeof(float)) != cudaSuccess) {
        h->det = nullptr;
        return det_fail(LBM_ERR_NOMEM, "set_more_details: device allocation failed");
    }
    if (cudaMalloc((void **)&h->stats, kStatFields * N * sizeof(double)) != cudaSuccess) {
        cudaFree(h->det);
        h->det = nullptr;
        h->stats = nullptr;
        return det_fail(LBM_ERR_NOMEM, "set_more_details: device allocation failed");
    }
    h->dev_bytes += kDetailFields * N * sizeof(float) + kStatFields * N * sizeof(double);
    if (cudaMemsetAsync(h->stats, 0, kStatFields * N * sizeof(double), h->s) != cudaSuccess ||
        cudaStreamSynchronize(h->s) != cudaSuccess)
        return det_fail(LBM_ERR_CUDA, "set_more_details: clearing the statistics failed");
    h->details = true;
    h->stat_samples = 0;
    h->stat_told = 0.0;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_sup_macroprop(lbm_handle *h, int n, int nt, double dt) {
    if (!h) return det_fail(LBM_ERR_INVALID, "sup_macroprop: null handle");
    if (!h->details) return det_fail(LBM_ERR_STATE, "sup_macroprop: call lbmgpu_set_more_details first");
    if (!h->inited) return det_fail(LBM_ERR_STATE, "sup_macroprop: call lbmgpu_init first");
    if (!(dt > 0.0)) return det_fail(LBM_ERR_INVALID, "sup_macroprop: dt must be positive");
    const double told = (double)(n - nt) * dt;
    if (told + dt == 0.0 || told + 1.0 == 0.0)
        return det_fail(LBM_ERR_INVALID, "sup_macroprop: (n - nt) dt is -dt or -1 (division by zero)");
    cudaError_t e = lbm_details_async(h, 1, told, dt);
    if (e != cudaSuccess) return det_fail(LBM_ERR_CUDA, std::string("sup_macroprop: ") + cudaGetErrorString(e));
    if (cudaStreamSynchronize(h->s) != cudaSuccess) return det_fail(LBM_ERR_CUDA, "sup_macroprop: sync failed");
    h->stat_samples++;
    h->stat_told = told;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download_details(lbm_handle *h, float *host) {
    if (!h || !host) return det_fail(LBM_ERR_INVALID, "download_details: null argument");
    if (!h->details) return det_fail(LBM_ERR_STATE, "download_details: call lbmgpu_set_more_details first");
    if (!h->inited) return det_fail(LBM_ERR_STATE, "download_details: call lbmgpu_init first");
    cudaError_t e = lbm_details_async(h, 0, 0.0, 1.0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host, h->det, (size_t)kDetailFields * det_cells(h) * sizeof(float),
                            cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return det_fail(LBM_ERR_CUDA, std::string("download_details: ") + cudaGetErrorString(e));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download_stats(lbm_handle *h, double *host, int *samples, double *told) {
    if (!h || !host) return det_fail(LBM_ERR_INVALID, "download_stats: null argument");
    if (!h->details) return det_fail(LBM_ERR_STATE, "download_stats: call lbmgpu_set_more_details first");
    cudaError_t e = cudaMemcpyAsync(host, h->stats, (size_t)kStatFields * det_cells(h) * sizeof(double),
                                    cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return det_fail(LBM_ERR_CUDA, std::string("download_stats: ") + cudaGetErrorString(e));
    if (samples) *samples = h->stat_samples;
    if (told) *told = h->stat_told;
    return LBM_OK;
}
