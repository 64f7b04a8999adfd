// lbm_batch.cu -- many independent lid-driven cavities of uneven sizes
// advanced together: one persistent launch per time step walks a flattened
// queue of cell tiles over all cavities (tile -> cavity through a table),
// and the host replays captured CUDA graphs of such launches.
//
// Each cavity is the reference's box with TYPE_S ghost walls and a moving
// lid on the ghost plane j = Ny+1 (as in lbm.cpp:1548-1551): per-cell wall
// velocity (Determine_Wall_Velocity, lbm.cpp:941-962) is the lid velocity
// for cells next to the lid plane and zero elsewhere, so the boundary links
// need no class table.  Populations are shifted (f - w), FP32 or FP16/BF16
// storage, FP32 arithmetic, one A/B pair per cavity inside one allocation.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_collide.cuh"
#include "lbm_device.cuh"

namespace lbmk {

struct BatchProb {
    int nx, ny, nz;
    int first;          // gather flag of the first step
    long long N;        // cells
    long long S;        // population stride
    long long base;     // element offset of population 0 in the A (and B) array
    long long mom_base; // offset of this cavity's moments in the moment array
    float omega;
    float lid;          // lid velocity along x
};

// tilexyz (optional): the (x, y | z << 16) of each tile's first cell, so a
// thread finds its cell by stepping along the rows instead of dividing.  A
// warp whose lanes all lie in rows off the y/z walls pulls plainly, the lanes
// on x = 0 / x = nx-1 bouncing back their x-crossing links (every row of a
// small cavity has two such lanes; a divergent boundary branch for them made
// every warp run both paths); warps touching a y/z wall take the per-link
// path.
template <class T, bool EXPORT>
__global__ void __launch_bounds__(512) k_batch_step(const T *__restrict__ A, T *__restrict__ B,
                                                    const BatchProb *__restrict__ probs,
                                                    const int2 *__restrict__ tiles, long long ntiles, int tile_cells,
                                                    int gather, uint32_t *__restrict__ status,
                                                    float *__restrict__ mom, const int2 *__restrict__ tilexyz) {
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tt = tiles[t];
        const BatchProb pr = probs[tt.x];
        const long long c = (long long)tt.y * tile_cells + threadIdx.x;
        const bool valid = threadIdx.x < tile_cells && c < pr.N;
        const int nx = pr.nx, ny = pr.ny, nz = pr.nz;
        const int cc = valid ? (int)c : 0;
        int x, y, z;
        if (tilexyz) {
            const int2 o = tilexyz[t];
            x = o.x + (int)threadIdx.x;
            y = o.y & 0xffff;
            z = o.y >> 16;
            while (x >= nx) {
                x -= nx;
                if (++y == ny) {
                    y = 0;
                    z++;
                }
            }
            if (!valid) x = y = z = 0;
        } else {
            x = cc % nx;
            y = (cc / nx) % ny;
            z = cc / (nx * ny);
        }
        const bool yzb = y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
        const bool bnd = yzb || x == 0 || x == nx - 1;
        const bool wyz = __any_sync(0xffffffffu, valid && yzb);
        const T *a = A + pr.base + cc;
        float f[Q];
        if (!gather) {
#pragma unroll
            for (int l = 0; l < Q; l++) f[l] = valid ? St<T>::ld(a + l * pr.S) : 0.0f;
        } else if (!wyz) {
            // rows off the y/z walls; x-face lanes bounce their x-crossing
            // links off the side walls (no lid there)
            // (the plain pull of an x-crossing link reads the neighbouring row's
            // end cell of the same population: inside the cavity's arrays,
            // since the cell's y and z are interior; then replaced)
#pragma unroll
            for (int l = 0; l < Q; l++)
                f[l] = valid ? St<T>::ld(a + l * pr.S - (cx(l) + nx * (cy(l) + ny * cz(l)))) : 0.0f;
            if (valid && (x == 0 || x == nx - 1)) {
                const bool xlo = x == 0;
#pragma unroll
                for (int l = 0; l < Q; l++)
                    if ((cx(l) > 0 && xlo) || (cx(l) < 0 && !xlo)) f[l] = St<T>::ld(a + opp(l) * pr.S);
            }
        } else if (!bnd) {
#pragma unroll
            for (int l = 0; l < Q; l++)
                f[l] = valid ? St<T>::ld(a + l * pr.S - (cx(l) + nx * (cy(l) + ny * cz(l)))) : 0.0f;
        } else {
            const bool lidcell = y == ny - 1;
#pragma unroll
            for (int l = 0; l < Q; l++) {
                float v = 0.0f;
                if (valid) {
                    const int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
                    if (sx < 0 || sx >= nx || sy < 0 || sy >= ny || sz < 0 || sz >= nz) {
                        // halfway bounce-back, moving-wall term 2 w (c.u_w) / cs^2 (lbm.cpp:274)
                        v = St<T>::ld(a + opp(l) * pr.S) + (lidcell ? 6.0f * wf(l) * cx(l) * pr.lid : 0.0f);
                    } else {
                        v = St<T>::ld(a + l * pr.S - (cx(l) + nx * (cy(l) + ny * cz(l))));
                    }
                }
                f[l] = v;
            }
        }
        float drho, jx, jy, jz;
        moments_pairs(f, drho, jx, jy, jz);
        const float rho = 1.0f + drho;
        const float inv = inv_one_plus(drho);
        const float ux = jx * inv, uy = jy * inv, uz = jz * inv;
        // one status update per warp (a warp lies in one tile, so one
        // cavity): a diverged cavity would otherwise send an atomic from
        // every cell of every step
        const unsigned badw = __ballot_sync(0xffffffffu, valid && !(rho > 0.0f && rho < 100.0f));
        if (badw && (threadIdx.x & 31) == 0) raise_status(&status[tt.x], ST_RHO_RANGE);
        if (EXPORT) {
            if (valid) {
                mom[pr.mom_base + cc] = rho;
                mom[pr.mom_base + pr.N + cc] = ux;
                mom[pr.mom_base + 2 * pr.N + cc] = uy;
                mom[pr.mom_base + 3 * pr.N + cc] = uz;
            }
            continue;
        }
        if (!valid) continue;
        collide_flow(f, drho, ux, uy, uz, 0.0f, 0.0f, 0.0f, false, pr.omega);
        T *b = B + pr.base + cc;
#pragma unroll
        for (int l = 0; l < Q; l++) St<T>::st(b + l * pr.S, f[l]);
    }
}

template <class T>
__global__ void k_batch_init(T *__restrict__ A, const BatchProb *__restrict__ probs, int nprob) {
    // f = feq(1, 0) shifted = 0 everywhere
    const int p = blockIdx.y;
    if (p >= nprob) return;
    const BatchProb pr = probs[p];
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < pr.N;
         c += (long long)gridDim.x * blockDim.x)
        for (int l = 0; l < Q; l++) St<T>::st(A + pr.base + l * pr.S + c, 0.0f);
}

}  // namespace lbmk

using namespace lbmk;

// error text shared with lbmgpu_last_error (lbm_abi.cu)
void lbm_set_last_error(const std::string &m);
static lbm_status bfail(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}
#define BCUDA(expr)                                                                                       \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)

struct lbm_batch {
    int n = 0;
    int storage = 0;
    size_t esize = 4;
    std::vector<BatchProb> hp;
    BatchProb *dp = nullptr;
    void *f[2] = {nullptr, nullptr};
    float *mom = nullptr;
    long long mom_total = 0;
    uint32_t *status = nullptr;
    int2 *tiles = nullptr;
    int2 *tilexyz = nullptr;  // first cell (x, y | z << 16) of each tile
    long long ntiles = 0;
    int tile_cells = 256;
    int grid = 0;
    int cur = 0;
    long long steps = 0;
    long long total_cells = 0;
    cudaStream_t s = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gsteps = 20;
};

template <class T>
static cudaError_t batch_launch(lbm_batch *b, int gather, bool exp) {
    const T *A = (const T *)b->f[b->cur];
    T *B = (T *)b->f[1 - b->cur];
    if (exp)
        k_batch_step<T, true><<<b->grid, b->tile_cells, 0, b->s>>>(A, B, b->dp, b->tiles, b->ntiles, b->tile_cells,
                                                                  gather, b->status, b->mom, b->tilexyz);
    else
        k_batch_step<T, false><<<b->grid, b->tile_cells, 0, b->s>>>(A, B, b->dp, b->tiles, b->ntiles, b->tile_cells,
                                                                   gather, b->status, nullptr, b->tilexyz);
    return cudaGetLastError();
}

static cudaError_t batch_enqueue(lbm_batch *b, int gather, bool exp) {
    switch (b->storage) {
    case 0: return batch_launch<float>(b, gather, exp);
    case 1: return batch_launch<__half>(b, gather, exp);
    case 2: return batch_launch<__nv_bfloat16>(b, gather, exp);
    }
    return cudaErrorInvalidValue;
}

static lbm_status batch_set_shape(lbm_batch *b, int tile_cells, int grid) {
    // tile table for this tile size
    std::vector<int2> t, txyz;
    for (int p = 0; p < b->n; p++) {
        const BatchProb &pr = b->hp[p];
        long long nt = (pr.N + tile_cells - 1) / tile_cells;
        for (long long k = 0; k < nt; k++) {
            t.push_back(make_int2(p, (int)k));
            const long long c0 = k * tile_cells;
            const int x0 = (int)(c0 % pr.nx), y0 = (int)((c0 / pr.nx) % pr.ny), z0 = (int)(c0 / ((long long)pr.nx * pr.ny));
            txyz.push_back(make_int2(x0, y0 | (z0 << 16)));
        }
    }
    if (b->tiles) cudaFree(b->tiles);
    if (b->tilexyz) cudaFree(b->tilexyz);
    b->tiles = nullptr;
    b->tilexyz = nullptr;
    BCUDA(cudaMalloc(&b->tiles, t.size() * sizeof(int2)));
    BCUDA(cudaMemcpyAsync(b->tiles, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice, b->s));
    // y and z each fit 16 bits (cavity edges are far below 65536)
    bool fits = true;
    for (int p = 0; p < b->n; p++) fits = fits && b->hp[p].ny < 65536 && b->hp[p].nz < 32768;
    if (fits) {
        BCUDA(cudaMalloc(&b->tilexyz, txyz.size() * sizeof(int2)));
        BCUDA(cudaMemcpyAsync(b->tilexyz, txyz.data(), txyz.size() * sizeof(int2), cudaMemcpyHostToDevice, b->s));
    }
    b->ntiles = (long long)t.size();
    b->tile_cells = tile_cells;
    b->grid = grid;
    for (int i = 0; i < 2; i++)
        if (b->gexec[i]) {
            cudaGraphExecDestroy(b->gexec[i]);
            b->gexec[i] = nullptr;
        }
    BCUDA(cudaStreamSynchronize(b->s));
    return LBM_OK;
}

static int persistent_grid(lbm_batch *b, int threads) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    switch (b->storage) {
    case 0: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<float, false>, threads, 0); break;
    case 1: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<__half, false>, threads, 0); break;
    default: cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<__nv_bfloat16, false>, threads, 0);
    }
    return std::max(1, per) * std::max(1, sms);
}

extern "C" lbm_status lbmgpu_batch_create(int n, const int *dims, const double *tau, double lid_u, int storage,
                                          lbm_batch **out) {
    if (!out || !dims || !tau || n < 1) return bfail(LBM_ERR_INVALID, "batch_create: bad arguments");
    if (storage < 0 || storage > 2) return bfail(LBM_ERR_INVALID, "batch_create: unknown storage");
    *out = nullptr;
    lbm_batch *b = new lbm_batch();
    b->n = n;
    b->storage = storage;
    b->esize = storage == 0 ? 4 : 2;
    long long base = 0, mb = 0;
    for (int p = 0; p < n; p++) {
        BatchProb pr;
        memset(&pr, 0, sizeof(pr));
        pr.nx = dims[3 * p];
        pr.ny = dims[3 * p + 1];
        pr.nz = dims[3 * p + 2];
        if (pr.nx < 2 || pr.ny < 2 || pr.nz < 2 || !(tau[p] > 0.5)) {
            delete b;
            return bfail(LBM_ERR_INVALID, "batch_create: cavity " + std::to_string(p) + " needs edges >= 2, tau > 0.5");
        }
        pr.N = (long long)pr.nx * pr.ny * pr.nz;
        pr.S = ((pr.N + 63) / 64) * 64;
        pr.base = base;
        pr.mom_base = mb;
        pr.omega = (float)(1.0 / tau[p]);
        pr.lid = (float)lid_u;
        base += (long long)Q * pr.S;
        mb += 4 * pr.N;
        b->total_cells += pr.N;
        b->hp.push_back(pr);
    }
    b->mom_total = mb;
    cudaError_t e = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking);
    for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaMalloc(&b->f[i], (size_t)base * b->esize);
    if (e == cudaSuccess) e = cudaMalloc(&b->mom, (size_t)mb * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&b->status, (size_t)n * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&b->dp, (size_t)n * sizeof(BatchProb));
    if (e == cudaSuccess) e = cudaMemcpy(b->dp, b->hp.data(), (size_t)n * sizeof(BatchProb), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->status, 0, (size_t)n * sizeof(uint32_t));
    for (int i = 0; i < 2 && e == cudaSuccess; i++) e = cudaEventCreate(&b->ev[i]);
    if (e != cudaSuccess) {
        lbm_status st = e == cudaErrorMemoryAllocation ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
        lbm_set_last_error(std::string("batch_create: ") + cudaGetErrorString(e));
        lbmgpu_batch_destroy(b);
        return st;
    }
    lbm_status st = batch_set_shape(b, 256, persistent_grid(b, 256));
    if (st != LBM_OK) {
        lbmgpu_batch_destroy(b);
        return st;
    }
    *out = b;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_destroy(lbm_batch *b) {
    if (!b) return LBM_OK;
    if (b->s) cudaStreamSynchronize(b->s);
    for (int i = 0; i < 2; i++) {
        if (b->gexec[i]) cudaGraphExecDestroy(b->gexec[i]);
        cudaFree(b->f[i]);
        if (b->ev[i]) cudaEventDestroy(b->ev[i]);
    }
    cudaFree(b->mom);
    cudaFree(b->status);
    cudaFree(b->dp);
    cudaFree(b->tiles);
    cudaFree(b->tilexyz);
    if (b->s) cudaStreamDestroy(b->s);
    delete b;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_init(lbm_batch *b) {
    if (!b) return bfail(LBM_ERR_INVALID, "batch_init: null");
    dim3 grd(256, b->n);
    switch (b->storage) {
    case 0: k_batch_init<float><<<grd, 256, 0, b->s>>>((float *)b->f[0], b->dp, b->n); break;
    case 1: k_batch_init<__half><<<grd, 256, 0, b->s>>>((__half *)b->f[0], b->dp, b->n); break;
    case 2: k_batch_init<__nv_bfloat16><<<grd, 256, 0, b->s>>>((__nv_bfloat16 *)b->f[0], b->dp, b->n); break;
    }
    BCUDA(cudaGetLastError());
    BCUDA(cudaMemsetAsync(b->status, 0, (size_t)b->n * sizeof(uint32_t), b->s));
    BCUDA(cudaStreamSynchronize(b->s));
    b->cur = 0;
    b->steps = 0;
    return LBM_OK;
}

static lbm_status batch_graph(lbm_batch *b) {
    const int p = b->cur;
    if (b->gexec[p]) return LBM_OK;
    cudaGraph_t g = nullptr;
    BCUDA(cudaStreamBeginCapture(b->s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < b->gsteps && e == cudaSuccess; i++) {
        e = batch_enqueue(b, 1, false);
        b->cur = 1 - b->cur;
    }
    cudaError_t e2 = cudaStreamEndCapture(b->s, &g);
    b->cur = p;
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return bfail(LBM_ERR_CUDA, "batch graph capture failed");
    }
    cudaError_t e3 = cudaGraphInstantiate(&b->gexec[p], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) return bfail(LBM_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e3));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_step(lbm_batch *b, int nsteps) {
    if (!b || nsteps < 0) return bfail(LBM_ERR_INVALID, "batch_step: bad arguments");
    while (nsteps > 0) {
        if (b->steps == 0) {
            BCUDA(batch_enqueue(b, 0, false));
            b->cur = 1 - b->cur;
            b->steps++;
            nsteps--;
            continue;
        }
        if (b->gsteps > 0 && nsteps >= b->gsteps) {
            lbm_status st = batch_graph(b);
            if (st != LBM_OK) return st;
            BCUDA(cudaGraphLaunch(b->gexec[b->cur], b->s));
            b->steps += b->gsteps;
            nsteps -= b->gsteps;
            continue;
        }
        BCUDA(batch_enqueue(b, 1, false));
        b->cur = 1 - b->cur;
        b->steps++;
        nsteps--;
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_step_timed(lbm_batch *b, int nsteps, double *ms) {
    if (!b || !ms) return bfail(LBM_ERR_INVALID, "batch_step_timed: null");
    BCUDA(cudaEventRecord(b->ev[0], b->s));
    lbm_status st = lbmgpu_batch_step(b, nsteps);
    if (st != LBM_OK) return st;
    BCUDA(cudaEventRecord(b->ev[1], b->s));
    BCUDA(cudaEventSynchronize(b->ev[1]));
    float t = 0.f;
    BCUDA(cudaEventElapsedTime(&t, b->ev[0], b->ev[1]));
    *ms = t;
    return LBM_OK;
}

// Autotuner: times each (threads per tile, persistent or one-tile-per-CTA
// grid) shape over a few graph replays and keeps the fastest.  The state
// advances meanwhile; callers re-initialise afterwards.
extern "C" lbm_status lbmgpu_batch_autotune(lbm_batch *b, int *chosen) {
    if (!b) return bfail(LBM_ERR_INVALID, "batch_autotune: null");
    const int cand_t[3] = {128, 256, 512};
    double best = 1e30;
    int bt = 256, bg = 0;
    for (int ti = 0; ti < 3; ti++)
        for (int persistent = 0; persistent < 2; persistent++) {
            const int threads = cand_t[ti];
            const long long nt = [&]() {
                long long s = 0;
                for (auto &p : b->hp) s += (p.N + threads - 1) / threads;
                return s;
            }();
            const int grid = persistent ? persistent_grid(b, threads) : (int)std::min<long long>(nt, 1ll << 30);
            lbm_status st = batch_set_shape(b, threads, grid);
            if (st != LBM_OK) return st;
            if ((st = lbmgpu_batch_step(b, b->gsteps + 1)) != LBM_OK) return st;  // warm + capture
            double ms = 0;
            if ((st = lbmgpu_batch_step_timed(b, 2 * b->gsteps, &ms)) != LBM_OK) return st;
            if (ms < best) {
                best = ms;
                bt = threads;
                bg = grid;
            }
        }
    lbm_status st = batch_set_shape(b, bt, bg);
    if (st != LBM_OK) return st;
    if (chosen) {
        chosen[0] = bt;
        chosen[1] = bg;
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_download(lbm_batch *b, int problem, float *host) {
    if (!b || !host || problem < 0 || problem >= b->n) return bfail(LBM_ERR_INVALID, "batch_download: bad arguments");
    BCUDA(batch_enqueue(b, b->steps == 0 ? 0 : 1, true));
    const BatchProb &pr = b->hp[problem];
    BCUDA(cudaMemcpyAsync(host, b->mom + pr.mom_base, (size_t)4 * pr.N * sizeof(float), cudaMemcpyDeviceToHost, b->s));
    BCUDA(cudaStreamSynchronize(b->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_status(lbm_batch *b, uint32_t *flags) {
    if (!b || !flags) return bfail(LBM_ERR_INVALID, "batch_status: null");
    BCUDA(cudaMemcpyAsync(flags, b->status, (size_t)b->n * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->s));
    BCUDA(cudaStreamSynchronize(b->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_batch_info(lbm_batch *b, long long *total_cells, long long *steps) {
    if (!b) return bfail(LBM_ERR_INVALID, "batch_info: null");
    if (total_cells) *total_cells = b->total_cells;
    if (steps) *steps = b->steps;
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// Batched cavities without any device allocation.
//
// Some callers cannot call cudaMalloc: a host that hands the solver buffers
// from its own pre-sized device pool and must stay inside that pool's fixed
// budget, or code that must not introduce the device-wide synchronisation an
// allocation can cause while other work is in flight.  For them this entry
// point runs k_batch_step on the caller's population buffers and keeps its
// own working data -- the per-cavity parameter table, the tile table and the
// per-cavity status words -- in one file-scope device array of fixed size.
// Every GPU that loads the library holds that array until the process exits.
// Every call shares it, so calls that overlap on the GPU race with each other.
// ---------------------------------------------------------------------------
namespace {
constexpr int kNoAllocMaxCavities = 1024;
constexpr long long kNoAllocMaxTiles = 1ll << 20;  // 256-cell tiles: up to 268M cells
constexpr int kNoAllocTile = 256;
struct NoAllocScratch {
    BatchProb prob[kNoAllocMaxCavities];
    uint32_t status[kNoAllocMaxCavities];
    int2 tiles[kNoAllocMaxTiles];
};
constexpr int kMaxDevices = 64;
}  // namespace

// 8.4 MB of working space
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];
static NoAllocScratch *g_noalloc_ptr[kMaxDevices];  // device address of the array, per device

extern "C" lbm_status lbmgpu_batch_step_noalloc(int n, const int *dims, const double *tau, double lid_u, int storage,
                                                void *pop_a, void *pop_b, int first_step, int nsteps,
                                                uint32_t *status_out, void *stream) {
    if (n < 1 || !dims || !tau || !pop_a || !pop_b || nsteps < 0 || storage < 0 || storage > 2)
        return bfail(LBM_ERR_INVALID, "batch_step_noalloc: bad arguments");
    if (n > kNoAllocMaxCavities)
        return bfail(LBM_ERR_INVALID, "batch_step_noalloc: " + std::to_string(n) + " cavities exceed the maximum of " +
                                          std::to_string(kNoAllocMaxCavities));
    std::vector<BatchProb> hp(n);
    std::vector<int2> tiles;
    long long base = 0;
    for (int p = 0; p < n; p++) {
        BatchProb &pr = hp[p];
        memset(&pr, 0, sizeof(pr));
        pr.nx = dims[3 * p];
        pr.ny = dims[3 * p + 1];
        pr.nz = dims[3 * p + 2];
        if (pr.nx < 2 || pr.ny < 2 || pr.nz < 2 || !(tau[p] > 0.5))
            return bfail(LBM_ERR_INVALID,
                         "batch_step_noalloc: cavity " + std::to_string(p) + " needs edges >= 2 and tau > 0.5");
        pr.N = (long long)pr.nx * pr.ny * pr.nz;
        pr.S = ((pr.N + 63) / 64) * 64;
        pr.base = base;
        pr.omega = (float)(1.0 / tau[p]);
        pr.lid = (float)lid_u;
        base += (long long)Q * pr.S;
        const long long nt = (pr.N + kNoAllocTile - 1) / kNoAllocTile;
        if ((long long)tiles.size() + nt > kNoAllocMaxTiles)
            return bfail(LBM_ERR_INVALID, "batch_step_noalloc: more than " + std::to_string(kNoAllocMaxTiles) +
                                              " tiles of 256 cells (" +
                                              std::to_string(kNoAllocMaxTiles * kNoAllocTile) + " cells) in total");
        for (long long k = 0; k < nt; k++) tiles.push_back(make_int2(p, (int)k));
    }
    int dev = 0;
    BCUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return bfail(LBM_ERR_UNSUPPORTED, "batch_step_noalloc: device index too large");
    if (!g_noalloc_ptr[dev]) {
        // once per device, with the device current: the device address of the
        // array (its host-side name is only a stand-in)
        void *p = nullptr;
        BCUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = reinterpret_cast<NoAllocScratch *>(p);
    }
    NoAllocScratch *sc = g_noalloc_ptr[dev];
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    // the tables are copied from this call's host vectors: a captured graph
    // would replay copies from freed host memory
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    BCUDA(cudaStreamIsCapturing(s, &cap));
    if (cap != cudaStreamCaptureStatusNone)
        return bfail(LBM_ERR_STATE, "batch_step_noalloc: not callable while the stream is being captured");
    BCUDA(cudaMemcpyAsync(sc->prob, hp.data(), (size_t)n * sizeof(BatchProb), cudaMemcpyHostToDevice, s));
    BCUDA(cudaMemcpyAsync(sc->tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, s));
    BCUDA(cudaMemsetAsync(sc->status, 0, (size_t)n * sizeof(uint32_t), s));  // starts at zero on every call
    int sms = 0, per = 0;
    BCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    switch (storage) {
    case 0: BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<float, false>, kNoAllocTile, 0)); break;
    case 1: BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<__half, false>, kNoAllocTile, 0)); break;
    default:
        BCUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_batch_step<__nv_bfloat16, false>, kNoAllocTile, 0));
    }
    const long long ntiles = (long long)tiles.size();
    const int grid = (int)std::min<long long>(ntiles, (long long)std::max(1, per) * std::max(1, sms));
    void *bufs[2] = {pop_a, pop_b};
    for (int i = 0; i < nsteps; i++) {
        const int gather = (i == 0 && first_step) ? 0 : 1;
        const void *A = bufs[i & 1];
        void *B = bufs[(i + 1) & 1];
        switch (storage) {
        case 0:
            k_batch_step<float, false><<<grid, kNoAllocTile, 0, s>>>((const float *)A, (float *)B, sc->prob, sc->tiles,
                                                                      ntiles, kNoAllocTile, gather, sc->status, nullptr,
                                                                      nullptr);
            break;
        case 1:
            k_batch_step<__half, false><<<grid, kNoAllocTile, 0, s>>>((const __half *)A, (__half *)B, sc->prob,
                                                                       sc->tiles, ntiles, kNoAllocTile, gather,
                                                                       sc->status, nullptr, nullptr);
            break;
        default:
            k_batch_step<__nv_bfloat16, false><<<grid, kNoAllocTile, 0, s>>>(
                (const __nv_bfloat16 *)A, (__nv_bfloat16 *)B, sc->prob, sc->tiles, ntiles, kNoAllocTile, gather,
                sc->status, nullptr, nullptr);
        }
        BCUDA(cudaGetLastError());
    }
    if (status_out) {
        BCUDA(cudaMemcpyAsync(status_out, sc->status, (size_t)n * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        BCUDA(cudaStreamSynchronize(s));
    }
    return LBM_OK;
}
