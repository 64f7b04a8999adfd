// lbm_checkpoint.cu -- save and restore the device state of a solve.
//
// The reference restarts by recomputing from its set-up; there is no state
// file.  A checkpoint here holds what the next step reads: the current
// population buffer (flow and heat), the device state word (step counters,
// band origin, FP64 rigid body), the markers (positions, desired velocity,
// marker density, force accumulators) and the force / momentum-exchange
// histories.  Restoring onto a handle created with the same configuration
// (and the same lbmgpu_set_markers / lbmgpu_set_solids calls) continues the
// run exactly where it was saved.  In MORE_DETAILS mode the Sup_MacroProp
// statistics (and their sample count and latest told) travel too; the
// restoring handle must be in that mode as well.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "lbm_handle.h"

namespace {

const char kMagic[8] = {'L', 'B', 'M', 'G', 'P', 'U', 'C', '2'};

struct CkptHeader {
    char magic[8];
    int nx, ny, nz, storage, thermal, ibm_markers, solids, details;
    long long S, steps, hist_cap, mea_cap;
    long long stat_samples;
    double stat_told;
};

lbm_status ck_fail(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

// One device region to or from the file.
struct Region {
    void *dev;
    size_t bytes;
};

std::vector<Region> regions(lbm_handle *h, int src_buffer) {
    std::vector<Region> r;
    const size_t pop = (size_t)lbmk::Q * h->P.S * h->esize;
    r.push_back({h->f[src_buffer], pop});
    if (h->cfg.thermal) r.push_back({h->g[src_buffer], (size_t)lbmk::QT * h->P.S * h->esize});
    r.push_back({h->ds, sizeof(DevState)});
    r.push_back({h->hist, (size_t)h->hist_cap * 8 * sizeof(double)});
    if (h->ibm) {
        const size_t n = (size_t)h->mk.n;
        r.push_back({h->mk.pos, 3 * n * sizeof(double)});
        r.push_back({h->mk.udes, 3 * n * sizeof(float)});
        r.push_back({h->mk.rho, n * sizeof(float)});
        r.push_back({h->mk.acc, 11 * n * sizeof(double)});
    }
    if (h->solids) r.push_back({h->mea_ring, (size_t)h->mea_cap * 4 * sizeof(double)});
    if (h->details) r.push_back({h->stats, (size_t)LBM_STAT_COUNT * h->P.N * sizeof(double)});
    return r;
}

CkptHeader header_of(lbm_handle *h) {
    CkptHeader c;
    memset(&c, 0, sizeof(c));
    memcpy(c.magic, kMagic, 8);
    c.nx = h->P.nx;
    c.ny = h->P.ny;
    c.nz = h->P.nz;
    c.storage = h->cfg.storage;
    c.thermal = h->cfg.thermal;
    c.ibm_markers = h->ibm ? h->mk.n : 0;
    c.solids = h->solids ? 1 : 0;
    c.details = h->details ? 1 : 0;
    c.stat_samples = h->stat_samples;
    c.stat_told = h->stat_told;
    c.S = h->P.S;
    c.steps = h->steps;
    c.hist_cap = h->hist_cap;
    c.mea_cap = h->mea_cap;
    return c;
}

// D2Q9 handles: a header of the configuration's shape and the step count,
// then the regions of l2d_checkpoint_regions.
const char kMagic2[8] = {'L', 'B', 'M', 'G', 'P', 'U', '2', 'D'};

struct Ckpt2Header {
    char magic[8];
    int shape[8];
    long long steps;
};

lbm_status save_2d(lbm_handle *h, const char *path) {
    if (!h->inited) return ck_fail(LBM_ERR_STATE, "save_state: call lbmgpu_init first");
    if (lbmgpu_sync(h) != LBM_OK) return LBM_ERR_CUDA;
    FILE *fp = fopen(path, "wb");
    if (!fp) return ck_fail(LBM_ERR_INVALID, std::string("save_state: cannot open ") + path);
    Ckpt2Header c;
    memset(&c, 0, sizeof(c));
    memcpy(c.magic, kMagic2, 8);
    l2d_checkpoint_shape(h, c.shape);
    c.steps = h->steps;
    bool ok = fwrite(&c, sizeof(c), 1, fp) == 1;
    std::vector<char> buf;
    for (const l2d_region &r : l2d_checkpoint_regions(h, -1)) {
        if (!ok) break;
        buf.resize(r.bytes);
        ok = cudaMemcpy(buf.data(), r.dev, r.bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
             fwrite(buf.data(), 1, r.bytes, fp) == r.bytes;
    }
    if (fclose(fp) != 0) ok = false;
    if (!ok) return ck_fail(LBM_ERR_CUDA, std::string("save_state: write failed: ") + path);
    return LBM_OK;
}

lbm_status load_2d(lbm_handle *h, const char *path) {
    if (lbmgpu_sync(h) != LBM_OK) return LBM_ERR_CUDA;
    FILE *fp = fopen(path, "rb");
    if (!fp) return ck_fail(LBM_ERR_INVALID, std::string("load_state: cannot open ") + path);
    Ckpt2Header c;
    int mine[8];
    l2d_checkpoint_shape(h, mine);
    if (fread(&c, sizeof(c), 1, fp) != 1 || memcmp(c.magic, kMagic2, 8) != 0) {
        fclose(fp);
        return ck_fail(LBM_ERR_INVALID, "load_state: not a D2Q9 state file");
    }
    if (memcmp(c.shape, mine, sizeof(mine)) != 0) {
        fclose(fp);
        return ck_fail(LBM_ERR_INVALID, "load_state: the file was saved from a different configuration");
    }
    std::vector<char> buf;
    bool ok = true;
    const std::vector<l2d_region> r0 = l2d_checkpoint_regions(h, 0), r1 = l2d_checkpoint_regions(h, 1);
    for (size_t i = 0; i < r0.size() && ok; i++) {
        buf.resize(r0[i].bytes);
        ok = fread(buf.data(), 1, r0[i].bytes, fp) == r0[i].bytes &&
             cudaMemcpy(r0[i].dev, buf.data(), r0[i].bytes, cudaMemcpyHostToDevice) == cudaSuccess;
        // both buffers alike: solid cells (never rewritten) read either
        if (ok && r0[i].both)
            ok = cudaMemcpy(r1[i].dev, buf.data(), r0[i].bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    fclose(fp);
    if (!ok) return ck_fail(LBM_ERR_INVALID, std::string("load_state: read failed: ") + path);
    return l2d_checkpoint_restored(h, c.steps);
}

}  // namespace

extern "C" lbm_status lbmgpu_save_state(lbm_handle *h, const char *path) {
    if (!h || !path) return ck_fail(LBM_ERR_INVALID, "save_state: null argument");
    if (h->d2) return save_2d(h, path);
    if (!h->inited) return ck_fail(LBM_ERR_STATE, "save_state: call lbmgpu_init first");
    if (lbmgpu_sync(h) != LBM_OK) return LBM_ERR_CUDA;
    FILE *fp = fopen(path, "wb");
    if (!fp) return ck_fail(LBM_ERR_INVALID, std::string("save_state: cannot open ") + path);
    const CkptHeader c = header_of(h);
    bool ok = fwrite(&c, sizeof(c), 1, fp) == 1;
    std::vector<char> buf;
    for (const Region &r : regions(h, h->cur)) {
        if (!ok) break;
        buf.resize(r.bytes);
        ok = cudaMemcpy(buf.data(), r.dev, r.bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
             fwrite(buf.data(), 1, r.bytes, fp) == r.bytes;
    }
    if (fclose(fp) != 0) ok = false;
    if (!ok) return ck_fail(LBM_ERR_CUDA, std::string("save_state: write failed: ") + path);
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_load_state(lbm_handle *h, const char *path) {
    if (!h || !path) return ck_fail(LBM_ERR_INVALID, "load_state: null argument");
    if (h->d2) return load_2d(h, path);
    if (lbmgpu_sync(h) != LBM_OK) return LBM_ERR_CUDA;
    FILE *fp = fopen(path, "rb");
    if (!fp) return ck_fail(LBM_ERR_INVALID, std::string("load_state: cannot open ") + path);
    CkptHeader c;
    const CkptHeader mine = header_of(h);
    if (fread(&c, sizeof(c), 1, fp) != 1 || memcmp(c.magic, kMagic, 8) != 0) {
        fclose(fp);
        return ck_fail(LBM_ERR_INVALID, "load_state: not a state file");
    }
    if (c.nx != mine.nx || c.ny != mine.ny || c.nz != mine.nz || c.storage != mine.storage ||
        c.thermal != mine.thermal || c.ibm_markers != mine.ibm_markers || c.solids != mine.solids ||
        c.details != mine.details ||
        c.S != mine.S || c.hist_cap != mine.hist_cap || c.mea_cap != mine.mea_cap) {
        fclose(fp);
        return ck_fail(LBM_ERR_INVALID, "load_state: the file was saved from a different configuration");
    }
    std::vector<char> buf;
    bool ok = true;
    for (const Region &r : regions(h, 0)) {
        buf.resize(r.bytes);
        ok = fread(buf.data(), 1, r.bytes, fp) == r.bytes &&
             cudaMemcpy(r.dev, buf.data(), r.bytes, cudaMemcpyHostToDevice) == cudaSuccess;
        if (!ok) break;
        // both buffers alike: solid cells (never rewritten) read either
        if (r.dev == h->f[0]) ok = cudaMemcpy(h->f[1], h->f[0], r.bytes, cudaMemcpyDeviceToDevice) == cudaSuccess;
        if (ok && h->cfg.thermal && r.dev == h->g[0])
            ok = cudaMemcpy(h->g[1], h->g[0], r.bytes, cudaMemcpyDeviceToDevice) == cudaSuccess;
        if (!ok) break;
    }
    fclose(fp);
    if (!ok) return ck_fail(LBM_ERR_INVALID, std::string("load_state: read failed: ") + path);
    h->cur = 0;
    h->steps = c.steps;
    h->stat_samples = (int)c.stat_samples;
    h->stat_told = c.stat_told;
    h->inited = true;
    for (int i = 0; i < 2; i++)
        if (h->gexec[i]) {
            cudaGraphExecDestroy(h->gexec[i]);
            h->gexec[i] = nullptr;
        }
    return LBM_OK;
}
