// lbm_abi.cu -- the extern "C" layer (include/lbmgpu.h): handles, device
// memory, boundary-class tables, step sequencing and CUDA-graph replay.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <cstddef>
#include <numeric>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_device.cuh"
#include "lbm_handle.h"
#include "lbm_internal.h"

using namespace lbmk;

static thread_local std::string g_err;
static constexpr size_t kGuard = 256;  // cells of slack before the first population array

static lbm_status fail(lbm_status s, const std::string &msg) {
    g_err = msg;
    return s;
}

void lbm_set_last_error(const std::string &m) { g_err = m; }

#define CUDA_TRY(expr)                                                                                    \
    do {                                                                                                  \
        cudaError_t e_ = (expr);                                                                          \
        if (e_ != cudaSuccess) return fail(LBM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
    } while (0)


// ---------------------------------------------------------------------------
// Boundary classes
// ---------------------------------------------------------------------------
static double feq3_host(double rho, const double u[3], int l) {
    const double cu = cx(l) * u[0] + cy(l) * u[1] + cz(l) * u[2];
    const double usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
    const double cs2 = 1.0 / 3.0;
    return rho * wd(l) *
           (1 + cu / cs2 + cu * cu / (2 * cs2 * cs2) - usq / (2 * cs2) + cu * cu * cu / (6 * cs2 * cs2 * cs2) -
            cu * usq / (2 * cs2 * cs2));
}

static int face_priority(int kind) {
    switch (kind) {
    case LBM_FACE_WALL: return 4;
    case LBM_FACE_INLET: return 3;
    case LBM_FACE_OUTLET_EQ: return 2;
    case LBM_FACE_OUTLET_ZG: return 1;
    }
    return 0;
}

// Faces crossed by offset d from a cell of class cls (non-periodic axes).
static int crossed_faces(int cls, const int d[3], int periodic, int faces_out[3]) {
    int n = 0;
    for (int a = 0; a < 3; a++) {
        if (periodic & (1 << a)) continue;
        if (d[a] < 0 && (cls & (1 << (2 * a)))) faces_out[n++] = 2 * a;
        if (d[a] > 0 && (cls & (1 << (2 * a + 1)))) faces_out[n++] = 2 * a + 1;
    }
    return n;
}

// The ghost cell reached across faces fs[0..n): highest-priority kind wins;
// for walls the velocity is that of a moving wall face among them (the last
// in x-, x+, y-, y+, z-, z+ order), else zero.
static int resolve_ghost(const lbm_config &c, const int *fs, int n, int *face_idx, double uw[3]) {
    int best = -1, bp = -1;
    for (int i = 0; i < n; i++) {
        int p = face_priority(c.faces[fs[i]].kind);
        if (p > bp) { bp = p; best = fs[i]; }
    }
    *face_idx = best;
    uw[0] = uw[1] = uw[2] = 0.0;
    if (best >= 0 && c.faces[best].kind == LBM_FACE_WALL) {
        for (int i = 0; i < n; i++) {
            const lbm_face &f = c.faces[fs[i]];
            if (f.kind != LBM_FACE_WALL) continue;
            if (f.u[0] != 0 || f.u[1] != 0 || f.u[2] != 0) { uw[0] = f.u[0]; uw[1] = f.u[1]; uw[2] = f.u[2]; }
        }
    }
    return best >= 0 ? c.faces[best].kind : -1;
}

static void build_classes(const lbm_config &c, StepParams &P) {
    for (int cls = 0; cls < 64; cls++) {
        ClassEntry e;
        memset(&e, 0, sizeof(e));
        // wall velocity of a cell of this class: mean over its moving wall
        // neighbours (Determine_Wall_Velocity, lbm.cpp:941-962)
        double uwall[3] = {0, 0, 0};
        int num = 0;
        for (int l = 0; l < Q; l++) {
            int d[3] = {cx(l), cy(l), cz(l)}, fs[3], fi;
            int n = crossed_faces(cls, d, P.periodic, fs);
            if (!n) continue;
            double uw[3];
            int kind = resolve_ghost(c, fs, n, &fi, uw);
            if (kind == LBM_FACE_WALL && (uw[0] != 0 || uw[1] != 0 || uw[2] != 0)) {
                uwall[0] += uw[0]; uwall[1] += uw[1]; uwall[2] += uw[2];
                num++;
            }
        }
        if (num) { uwall[0] /= num; uwall[1] /= num; uwall[2] /= num; }
        for (int l = 0; l < Q; l++) {
            int d[3] = {-cx(l), -cy(l), -cz(l)}, fs[3], fi;
            int n = crossed_faces(cls, d, P.periodic, fs);
            if (!n) continue;
            double uw[3];
            int kind = resolve_ghost(c, fs, n, &fi, uw);
            const lbm_face &F = c.faces[fi];
            if (kind == LBM_FACE_WALL) {
                e.bb |= 1u << l;
                // f_l(x) = f*_opp(l)(x) - 2 w (u_w . c_opp) / cs^2 (lbm.cpp:274)
                e.val[l] = (float)(6.0 * wd(l) * (uwall[0] * cx(l) + uwall[1] * cy(l) + uwall[2] * cz(l)));
                if (l < QT && F.thermal_kind == LBM_TWALL_DIRICHLET) {
                    e.tdir |= 1u << l;
                    e.tval[l] = (float)(2.0 * (l == 0 ? 0.25 : 0.125) * F.T);
                }
            } else if (kind == LBM_FACE_INLET || kind == LBM_FACE_OUTLET_EQ) {
                e.eq |= 1u << l;
                e.val[l] = (float)(feq3_host(F.rho, F.u, l) - wd(l));
                if (l < QT) {
                    const double cu = cx(l) * F.u[0] + cy(l) * F.u[1] + cz(l) * F.u[2];
                    e.tval[l] = (float)((l == 0 ? 0.25 : 0.125) * F.T * (1.0 + 4.0 * cu));
                }
            } else if (kind == LBM_FACE_OUTLET_ZG) {
                e.zg |= 1u << l;
            }
        }
        P.cls[cls] = e;
    }
}

// The x-face table (XFix) of rows off the y/z faces: what the boundary-class
// rule of pull_link / pull_heat_link gives for the five x-crossing links of a
// cell on x = 0 (face 0) and x = nx-1 (face 1), as an offset from the cell,
// a factor and a constant.
static void build_xfix(StepParams &P) {
    const int pm = ((P.periodic & 1) ? 3 : 0) | ((P.periodic & 2) ? 12 : 0) | ((P.periodic & 4) ? 48 : 0);
    for (int f = 0; f < 2; f++) {
        XFix &xf = P.xf[f];
        memset(&xf, 0, sizeof(xf));
        const ClassEntry &ce = P.cls[(f == 0 ? 1 : 2) & ~pm];
        const int x = f == 0 ? 0 : P.nx - 1;
        auto pull_ofs = [&](int l) -> long long {
            int sx = x - cx(l);
            if (P.periodic & 1) sx = sx < 0 ? sx + P.nx : (sx >= P.nx ? sx - P.nx : sx);
            if ((ce.zg >> l) & 1u) sx = std::min(std::max(sx, 0), P.nx - 1);
            return (long long)l * P.S + (sx - x) - (long long)P.nx * (cy(l) + (long long)P.ny * cz(l));
        };
        for (int k = 0; k < 5; k++) {
            const int l = f == 0 ? lbmk::xpl(k) : lbmk::xml(k);
            if ((ce.bb >> l) & 1u) {
                xf.ofs[k] = (unsigned)((long long)opp(l) * P.S);
                xf.sgn[k] = 1.0f;
                xf.add[k] = ce.val[l];
            } else if ((ce.eq >> l) & 1u) {
                xf.eq |= 1u << k;
                xf.ofs[k] = (unsigned)((long long)l * P.S);
                xf.add[k] = ce.val[l];
            } else {
                xf.ofs[k] = (unsigned)pull_ofs(l);
                xf.sgn[k] = 1.0f;
                xf.add[k] = 0.0f;
            }
        }
        const int lt = f == 0 ? 1 : 2;  // the D3Q7 link across this face
        if ((ce.bb >> lt) & 1u) {
            const bool dir = (ce.tdir >> lt) & 1u;
            xf.tofs = (unsigned)((long long)opp(lt) * P.S);
            xf.tsgn = dir ? -1.0f : 1.0f;
            xf.tadd = dir ? ce.tval[lt] : 0.0f;
        } else if ((ce.eq >> lt) & 1u) {
            xf.teq = 1;
            xf.tofs = (unsigned)((long long)lt * P.S);
            xf.tadd = ce.tval[lt];
        } else {
            xf.tofs = (unsigned)pull_ofs(lt);
            xf.tsgn = 1.0f;
        }
    }
}

// Default thread block: 128 x 2 for FP32 storage, 128 x 1 for FP16/BF16.
// The half-storage kernel is issue-bound; its 128-thread blocks packed
// beside the IBM phase's kernels ran the 256x128x128 sphere 2.8 % faster
// (40.7 k against 39.5 k MLUPS), while FP32 changed by about 1 % between
// the shapes tried.
static void choose_block(lbm_handle *h) {
    int nx = h->cfg.nx;
    int tx = h->cfg.block_x, ty = h->cfg.block_y;
    if (tx <= 0) tx = nx >= 128 ? 128 : (nx >= 64 ? 64 : 32);
    const int threads = h->cfg.storage == LBM_STORE_F32 ? 256 : 128;
    if (ty <= 0) ty = std::max(1, threads / tx);
    if (tx % 32 != 0) tx = ((tx + 31) / 32) * 32;
    h->tx = tx;
    h->ty = ty;
}

// ---------------------------------------------------------------------------
// Creation
// ---------------------------------------------------------------------------
extern "C" int lbmgpu_abi_version(void) { return 3; }

cudaStream_t lbm_handle_stream(lbm_handle *h) { return h->s; }

extern "C" const char *lbmgpu_last_error(void) { return g_err.c_str(); }

extern "C" lbm_status lbmgpu_config_from_types(int nx, int ny, int nz, double tau, const uint8_t *types,
                                               const double *rho, const double *ux, const double *uy,
                                               const double *uz, const double *T, lbm_config *out) {
    if (!types || !out || nx < 1 || ny < 1 || nz < 1) return fail(LBM_ERR_INVALID, "config_from_types: bad arguments");
    const int NX = nx + 2, NY = ny + 2;
    auto at = [&](int i, int j, int k) { return (size_t)i + (size_t)NX * ((size_t)j + (size_t)NY * k); };
    lbm_config c;
    memset(&c, 0, sizeof(c));
    c.tau = tau;
    c.rho0 = 1.0;
    // interior: fluid, or solid at rest (lbmgpu_set_solids)
    for (int k = 1; k <= nz; k++)
        for (int j = 1; j <= ny; j++)
            for (int i = 1; i <= nx; i++) {
                const size_t c = at(i, j, k);
                if (types[c] == 0) continue;
                if (types[c] != 1)
                    return fail(LBM_ERR_UNSUPPORTED, "config_from_types: non-fluid cell inside the domain");
                if ((ux && ux[c] != 0) || (uy && uy[c] != 0) || (uz && uz[c] != 0))
                    return fail(LBM_ERR_UNSUPPORTED, "config_from_types: moving solid cell inside the domain");
            }
    // face planes (without edges): uniform type and state
    const int lim[3] = {nx, ny, nz};
    int periodic_axis[3] = {0, 0, 0};
    for (int f = 0; f < 6; f++) {
        int a = f / 2, side = f % 2;
        int fixed = side ? lim[a] + 1 : 0;
        int b = (a + 1) % 3, cc = (a + 2) % 3;
        int kind0 = -1;
        double st[5] = {0, 0, 0, 0, 0};
        for (int p = 1; p <= lim[b]; p++)
            for (int q = 1; q <= lim[cc]; q++) {
                int ijk[3];
                ijk[a] = fixed;
                ijk[b] = p;
                ijk[cc] = q;
                size_t id = at(ijk[0], ijk[1], ijk[2]);
                int t = types[id];
                double s[5] = {rho ? rho[id] : 1.0, ux ? ux[id] : 0.0, uy ? uy[id] : 0.0, uz ? uz[id] : 0.0,
                               T ? T[id] : 0.0};
                if (kind0 < 0) {
                    kind0 = t;
                    memcpy(st, s, sizeof(st));
                } else if (t != kind0 || memcmp(st, s, sizeof(st)) != 0) {
                    return fail(LBM_ERR_UNSUPPORTED, "config_from_types: face " + std::to_string(f) + " is not uniform");
                }
            }
        lbm_face &F = c.faces[f];
        F.rho = st[0];
        F.u[0] = st[1];
        F.u[1] = st[2];
        F.u[2] = st[3];
        F.T = st[4];
        switch (kind0) {
        case 1: F.kind = LBM_FACE_WALL; break;       // TYPE_S
        case 3: F.kind = LBM_FACE_INLET; break;      // TYPE_IN
        case 2: F.kind = LBM_FACE_OUTLET_EQ; break;  // TYPE_OUT
        case 0: F.kind = LBM_FACE_PERIODIC; periodic_axis[a]++; break;  // TYPE_F ghost: wraps
        default: return fail(LBM_ERR_UNSUPPORTED, "config_from_types: unsupported ghost type " + std::to_string(kind0));
        }
    }
    int dims[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++) {
        if (periodic_axis[a] == 1) return fail(LBM_ERR_UNSUPPORTED, "config_from_types: one-sided TYPE_F ghost face");
        if (periodic_axis[a] == 2) dims[a] += 2;  // the reference wraps over N+2 cells
    }
    c.nx = dims[0];
    c.ny = dims[1];
    c.nz = dims[2];
    *out = c;
    return LBM_OK;
}

static void free_handle(lbm_handle *h) {
    if (!h) return;
    if (h->d2) l2d_free(h);
    for (int i = 0; i < 2; i++) {
        if (h->gexec[i]) cudaGraphExecDestroy(h->gexec[i]);
        if (h->fraw[i]) cudaFree(h->fraw[i]);
        if (h->graw[i]) cudaFree(h->graw[i]);
    }
    cudaFree(h->mom);
    cudaFree(h->band);
    cudaFree(h->nu_scratch);
    cudaFree(h->ds);
    cudaFree(h->hist);

    cudaFree(h->mk.pos);
    cudaFree(h->mk.ds);
    cudaFree(h->mk.udes);
    cudaFree(h->mk.rho);
    cudaFree(h->mk.force);
    cudaFree(h->mk.acc);
    cudaFree(h->mk.sb);
    cudaFree(h->mk.sw);
    cudaFree(h->mk.ipart);
    for (int i = 0; i < 4; i++)
        if (h->ev[i]) cudaEventDestroy(h->ev[i]);
    for (cudaEvent_t e : h->evpool) cudaEventDestroy(e);
    if (h->ev_near) cudaEventDestroy(h->ev_near);
    lbm_output_free(h);
    for (void *p : {(void *)h->solid_d, (void *)h->near_d, (void *)h->mea_part, (void *)h->mea_blocks,
                    (void *)h->mea_ring, (void *)h->det, (void *)h->stats})
        if (p) cudaFree(p);
    if (h->ev_ibm) cudaEventDestroy(h->ev_ibm);
    if (h->ev_acc) cudaEventDestroy(h->ev_acc);
    if (h->ev_fin) cudaEventDestroy(h->ev_fin);
    if (h->s_dl) cudaStreamSynchronize(h->s_dl);
    if (h->ev_dl_exported) cudaEventDestroy(h->ev_dl_exported);
    if (h->ev_dl_copied) cudaEventDestroy(h->ev_dl_copied);
    if (h->s_dl) cudaStreamDestroy(h->s_dl);
    if (h->s2) cudaStreamDestroy(h->s2);
    if (h->s3) cudaStreamDestroy(h->s3);
    if (h->s) cudaStreamDestroy(h->s);
    if (h->fstage) cudaFreeHost(h->fstage);
    delete h;
}

template <class Tp>
static cudaError_t dalloc(lbm_handle *h, Tp **p, size_t bytes) {
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e == cudaSuccess) h->dev_bytes += bytes;
    return e;
}

extern "C" lbm_status lbmgpu_create(const lbm_config *cfg, lbm_handle **out) {
    if (!cfg || !out) return fail(LBM_ERR_INVALID, "create: null argument");
    *out = nullptr;
    const lbm_config &c = *cfg;
    if (c.nx < 1 || c.ny < 1 || c.nz < 1) return fail(LBM_ERR_INVALID, "create: grid extents must be >= 1");
    if (!(c.tau > 0.5)) return fail(LBM_ERR_INVALID, "create: tau must be > 0.5 (nu = (tau - 0.5)/3 > 0)");
    if (c.storage < 0 || c.storage > 2) return fail(LBM_ERR_INVALID, "create: unknown storage format");
    if (c.thermal && !(c.tau_g > 0.5)) return fail(LBM_ERR_INVALID, "create: tau_g must be > 0.5");
    for (int a = 0; a < 3; a++) {
        bool p0 = c.faces[2 * a].kind == LBM_FACE_PERIODIC, p1 = c.faces[2 * a + 1].kind == LBM_FACE_PERIODIC;
        if (p0 != p1) return fail(LBM_ERR_INVALID, "create: a periodic axis needs both faces periodic");
    }
    for (int f = 0; f < 6; f++)
        if (c.faces[f].kind < 0 || c.faces[f].kind > 4) return fail(LBM_ERR_INVALID, "create: unknown face kind");
    if (c.lattice != 0 && c.lattice != LBM_LATTICE_D3Q19 && c.lattice != LBM_LATTICE_D2Q9)
        return fail(LBM_ERR_INVALID, "create: unknown lattice");
    if (c.staged > 0)
        return fail(LBM_ERR_UNSUPPORTED, "create: the staged (tensor-copy) step kernel is not built (staged must be 0)");
    if (c.wall_force && c.lattice != LBM_LATTICE_D2Q9)
        return fail(LBM_ERR_UNSUPPORTED, "create: wall_force is a D2Q9 option (the reference's Poiseuille_Flow)");
    if (c.thermal < LBM_THERMAL_NONE || c.thermal > LBM_THERMAL_ENERGY)
        return fail(LBM_ERR_INVALID, "create: unknown thermal model");
    if (c.lattice != LBM_LATTICE_D2Q9 && c.thermal == LBM_THERMAL_ENERGY)
        return fail(LBM_ERR_UNSUPPORTED, "create: the ENERGY model on D3Q19 is its own solver object "
                                         "(lbmgpu_energy3d_create)");
    for (int f = 0; f < 6; f++)
        if (c.lattice != LBM_LATTICE_D2Q9 && c.faces[f].kind == LBM_FACE_WALL &&
            c.faces[f].thermal_kind == LBM_TWALL_NEUMANN)
            return fail(LBM_ERR_UNSUPPORTED, "create: Neumann thermal walls are a D2Q9 ENERGY option");
    if (c.lattice == LBM_LATTICE_D2Q9) {
        lbm_handle *h = new lbm_handle();
        h->cfg = c;
        lbm_status st = l2d_create(h);
        for (int i = 0; i < 4 && st == LBM_OK; i++)
            if (cudaEventCreate(&h->ev[i]) != cudaSuccess) st = fail(LBM_ERR_CUDA, "create: events");
        if (st != LBM_OK) {
            free_handle(h);
            return st;
        }
        *out = h;
        return LBM_OK;
    }
    lbm_handle *h = new lbm_handle();
    h->cfg = c;
    memset(&h->P, 0, sizeof(h->P));
    StepParams &P = h->P;
    P.nx = c.nx;
    P.ny = c.ny;
    P.nz = c.nz;
    P.N = (long long)c.nx * c.ny * c.nz;
    for (int a = 0; a < 3; a++)
        if (c.faces[2 * a].kind == LBM_FACE_PERIODIC) P.periodic |= 1 << a;
    P.omega = (float)(1.0 / c.tau);
    P.omega_t = c.thermal ? (float)(1.0 / c.tau_g) : 0.0f;
    for (int a = 0; a < 3; a++) {
        P.body[a] = (float)c.body_force[a];
        P.gbeta[a] = c.thermal ? (float)c.gbeta[a] : 0.0f;
    }
    P.T0 = (float)c.T_ref;
    P.forced = (c.body_force[0] != 0 || c.body_force[1] != 0 || c.body_force[2] != 0 ||
                (c.thermal && (c.gbeta[0] != 0 || c.gbeta[1] != 0 || c.gbeta[2] != 0)))
                   ? 1
                   : 0;
    build_classes(c, P);
    h->esize = c.storage == LBM_STORE_F32 ? 4 : 2;
    if (c.graph_steps > 0) h->gsteps = c.graph_steps + (c.graph_steps & 1);
    if (c.graph_steps < 0) h->gsteps = 0;
    choose_block(h);
    lbm_status st = LBM_OK;
    auto chk = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == LBM_OK) {
            st = (e == cudaErrorMemoryAllocation) ? LBM_ERR_NOMEM : LBM_ERR_CUDA;
            g_err = std::string("create: ") + what + ": " + cudaGetErrorString(e);
        }
    };
    chk(cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking), "stream");
    // Population arrays: stride S = N plus at least two rows (and 512 cells)
    // of slack, rounded up to 256 cells, so that every speculative read (idle
    // lanes, a row segment's edge word one row past the last plane) stays
    // inside the array, and a guard of kGuard cells before the first array.
    P.S = ((P.N + std::max<long long>(512, 2LL * P.nx + 64) + 255) / 256) * 256;
    for (int l = 0; l < Q; l++)
        P.pofs[l] = (long long)l * P.S - ((long long)cx(l) + (long long)P.nx * ((long long)cy(l) + (long long)P.ny * cz(l)));
    // 32-bit element indices: every index (cell + l S - shift) stays below
    // 19 S < 2^31 and is never negative (S exceeds any shift); idle lanes
    // load the stencil of cell (1,1,1), which needs every edge >= 3
    P.idx32 = ((long long)Q * P.S + P.nx * (long long)P.ny < (1LL << 31) && P.nx >= 3 && P.ny >= 3 && P.nz >= 3 &&
               P.S > 1 + (long long)P.nx + (long long)P.nx * P.ny)
                  ? 1
                  : 0;
    P.safe_cell = P.idx32 ? (unsigned)(1 + P.nx * (1 + (long long)P.ny)) : 0u;
    for (int l = 0; l < Q; l++) {
        P.pofs32[l] = P.idx32 ? (unsigned)P.pofs[l] : 0u;
        P.sofs32[l] = P.idx32 ? (unsigned)((long long)l * P.S) : 0u;
        P.rofs32[l] = P.idx32 ? (unsigned)((long long)l * P.S - (long long)P.nx * ((long long)cy(l) + (long long)P.ny * cz(l)))
                              : 0u;
    }
    // x-face lanes fix their own x-crossing links: warps stay on the plain
    // pull in every row that is not on a y/z face
    P.xface = (c.xface >= 0 && P.nx >= 2 && P.ny >= 3 && P.nz >= 3) ? 1 : 0;
    if (P.idx32) build_xfix(P);
    {
        // two x-cells per thread (packed pair arithmetic) for FP16/BF16 storage
        // on lattices of 2^20 cells or more; one for FP32, which is
        // memory-bound with one cell per thread, and for smaller lattices,
        // which sit in L2 and are bound by latency: a 64^3 FP16 cavity ran
        // 20.1 k MLUPS with one cell a thread against 17.6 k with two, a 128^3
        // one 43.2 k against 44.7 k, the 256 x 128 x 128 one 50.9 k against 54.1 k
        const bool big = (long long)P.nx * P.ny * P.nz >= (1LL << 20);
        const int v = c.cells_per_thread > 0 ? c.cells_per_thread : (c.storage == LBM_STORE_F32 || !big ? 1 : 2);
        h->vcells = (v > 1 && lbmk::step_vec_usable(c.storage, P, v)) ? v : 0;
    }
    const size_t fb = ((size_t)Q * P.S + 2 * kGuard) * h->esize;
    for (int i = 0; i < 2 && st == LBM_OK; i++) {
        chk(dalloc(h, &h->fraw[i], fb), "populations");
        if (st == LBM_OK) h->f[i] = (char *)h->fraw[i] + kGuard * h->esize;
    }
    if (c.thermal)
        for (int i = 0; i < 2 && st == LBM_OK; i++) {
            chk(dalloc(h, &h->graw[i], ((size_t)QT * P.S + 2 * kGuard) * h->esize), "thermal");
            if (st == LBM_OK) h->g[i] = (char *)h->graw[i] + kGuard * h->esize;
        }
    // moments: rho, u (3) [, T, heat flux (3)]
    if (st == LBM_OK) chk(dalloc(h, &h->mom, (size_t)(c.thermal ? 8 : 5) * P.N * sizeof(float)), "moments");
    if (st == LBM_OK) chk(dalloc(h, &h->ds, sizeof(DevState)), "state");
    if (st == LBM_OK) chk(dalloc(h, &h->hist, (size_t)h->hist_cap * 8 * sizeof(double)), "history");
    if (st == LBM_OK) {
        DevState d;
        memset(&d, 0, sizeof(d));
        d.hist_cap = h->hist_cap;
        chk(cudaMemcpyAsync(h->ds, &d, sizeof(d), cudaMemcpyHostToDevice, h->s), "state init");
        chk(cudaMemsetAsync(h->hist, 0, (size_t)h->hist_cap * 8 * sizeof(double), h->s), "history init");
    }
    for (int i = 0; i < 4 && st == LBM_OK; i++) chk(cudaEventCreate(&h->ev[i]), "events");
    if (st == LBM_OK) {
        int lo = 0, hi = 0;
        chk(cudaDeviceGetStreamPriorityRange(&lo, &hi), "priority range");
        chk(cudaStreamCreateWithPriority(&h->s2, cudaStreamNonBlocking, hi), "ibm stream");
        chk(cudaEventCreateWithFlags(&h->ev_near, cudaEventDisableTiming), "events");
        chk(cudaStreamCreateWithPriority(&h->s3, cudaStreamNonBlocking, hi), "reduction stream");
        chk(cudaEventCreateWithFlags(&h->ev_ibm, cudaEventDisableTiming), "events");
        chk(cudaEventCreateWithFlags(&h->ev_acc, cudaEventDisableTiming), "events");
        chk(cudaEventCreateWithFlags(&h->ev_fin, cudaEventDisableTiming), "events");
        if (st == LBM_OK) chk(cudaEventRecord(h->ev_ibm, h->s), "events");
        if (st == LBM_OK) chk(cudaEventRecord(h->ev_fin, h->s), "events");
    }
    if (st == LBM_OK) chk(cudaStreamSynchronize(h->s), "sync");
    if (st != LBM_OK) {
        free_handle(h);
        return st;
    }
    *out = h;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_destroy(lbm_handle *h) {
    if (!h) return LBM_OK;
    if (h->s2) cudaStreamSynchronize(h->s2);
    if (h->s3) cudaStreamSynchronize(h->s3);
    if (h->s) cudaStreamSynchronize(h->s);
    free_handle(h);
    return LBM_OK;
}

static lbm_status do_init(lbm_handle *h, const float *dfields) {
    float init[5] = {(float)h->cfg.rho0, (float)h->cfg.u0[0], (float)h->cfg.u0[1], (float)h->cfg.u0[2],
                     (float)h->cfg.T_init};
    // with solid cells both buffers start alike: a solid cell is never
    // rewritten and keeps its initial populations in A and B
    CUDA_TRY(launch_init(h->cfg.storage, h->f[0], h->g[0], h->solids ? h->f[1] : nullptr,
                         h->solids ? h->g[1] : nullptr, h->P.N, h->P.S, dfields, init, h->cfg.thermal != 0, h->s));
    if (h->solids) {
        // the first momentum-exchange record is that of reference step 1
        const long long one = 1;
        CUDA_TRY(cudaMemcpyAsync((char *)h->ds + offsetof(DevState, mea_step), &one, sizeof(one),
                                 cudaMemcpyHostToDevice, h->s));
    }
    h->cur = 0;
    h->steps = 0;
    h->inited = true;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_init(lbm_handle *h) {
    if (!h) return fail(LBM_ERR_INVALID, "init: null handle");
    if (h->d2) return l2d_init(h, nullptr, nullptr, nullptr);
    lbm_status s = do_init(h, nullptr);
    if (s != LBM_OK) return s;
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_init_fields(lbm_handle *h, const double *rho, const double *ux, const double *uy,
                                         const double *uz, const double *T) {
    if (!h || !rho || !ux || !uy || !uz) return fail(LBM_ERR_INVALID, "init_fields: null argument");
    if (h->d2) return l2d_init(h, rho, ux, uy);
    const long long N = h->P.N;
    std::vector<float> tmp((size_t)5 * N);
    for (long long c = 0; c < N; c++) {
        tmp[c] = (float)rho[c];
        tmp[N + c] = (float)ux[c];
        tmp[2 * N + c] = (float)uy[c];
        tmp[3 * N + c] = (float)uz[c];
        tmp[4 * N + c] = T ? (float)T[c] : (float)h->cfg.T_init;
    }
    // the moment buffer doubles as upload staging
    CUDA_TRY(lbm_mom_acquire(h));
    CUDA_TRY(cudaMemcpyAsync(h->mom, tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice, h->s));
    lbm_status s = do_init(h, h->mom);
    if (s != LBM_OK) return s;
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// IBM set-up
// ---------------------------------------------------------------------------
extern "C" lbm_status lbmgpu_set_markers(lbm_handle *h, const lbm_ibm_config *ic, const double *xyz, const double *ds,
                                         const double *udes) {
    if (!h || !ic || !xyz || !ds) return fail(LBM_ERR_INVALID, "set_markers: null argument");
    if (h->d2) return l2d_set_markers(h, ic, xyz, ds);
    if (ic->n_markers < 1 || ic->m_max < 1) return fail(LBM_ERR_INVALID, "set_markers: need markers and m_max >= 1");
    if (!(ic->radius > 0)) return fail(LBM_ERR_INVALID, "set_markers: radius must be > 0");
    if (ic->free_body && (!(ic->density_ratio > 0.0) || !(ic->volume > 0.0) || !(ic->inertia > 0.0)))
        return fail(LBM_ERR_INVALID, "set_markers: free body needs density_ratio, volume and inertia > 0");
    if (ic->thermal && !h->cfg.thermal) return fail(LBM_ERR_INVALID, "set_markers: thermal IBM needs a thermal lattice");
    const int n = ic->n_markers;
    const bool fresh = !h->ibm || h->mk.n != n;
    if (fresh) {
        cudaFree(h->mk.pos);
        cudaFree(h->mk.ds);
        cudaFree(h->mk.udes);
        cudaFree(h->mk.rho);
        cudaFree(h->mk.force);
        cudaFree(h->mk.acc);
        cudaFree(h->mk.sb);
        cudaFree(h->mk.sw);
        cudaFree(h->mk.ipart);
        cudaFree(h->band);
        memset(&h->mk, 0, sizeof(h->mk));
        h->band = nullptr;
        CUDA_TRY(dalloc(h, &h->mk.pos, (size_t)3 * n * sizeof(double)));
        CUDA_TRY(dalloc(h, &h->mk.ds, (size_t)n * sizeof(double)));
        CUDA_TRY(dalloc(h, &h->mk.udes, (size_t)3 * n * sizeof(float)));
        CUDA_TRY(dalloc(h, &h->mk.rho, (size_t)n * sizeof(float)));
        CUDA_TRY(dalloc(h, &h->mk.force, (size_t)4 * n * sizeof(float)));
        CUDA_TRY(dalloc(h, &h->mk.acc, (size_t)11 * n * sizeof(double)));
        CUDA_TRY(dalloc(h, &h->mk.sb, (size_t)3 * n * sizeof(int)));
        CUDA_TRY(dalloc(h, &h->mk.sw, (size_t)12 * n * sizeof(float)));
        CUDA_TRY(dalloc(h, &h->mk.ipart, (size_t)6 * lbmk::kBodyBlocks * sizeof(double)));
        h->mk.n = n;
    }
    h->icfg = *ic;
    h->mk.tdes = (float)ic->T_body;
    // band: every stencil node of a marker within `radius` of the centre
    int bs[3], dims[3] = {h->P.nx, h->P.ny, h->P.nz}, org[3];
    for (int a = 0; a < 3; a++) {
        bs[a] = std::min(dims[a], (int)std::ceil(2.0 * ic->radius) + 6);
        int o = (int)std::floor(ic->center[a] - ic->radius) - 2;
        org[a] = std::max(0, std::min(o, dims[a] - bs[a]));
    }
    long long nb = (long long)bs[0] * bs[1] * bs[2];
    if (fresh || nb != h->P.nb) {
        cudaFree(h->band);
        h->band = nullptr;
        // 12 FP32 arrays, then the 4 fixed-point force/heat accumulators
        CUDA_TRY(dalloc(h, &h->band, (size_t)12 * nb * sizeof(float) + (size_t)4 * nb * sizeof(long long)));
        CUDA_TRY(cudaMemsetAsync(h->band, 0, (size_t)12 * nb * sizeof(float) + (size_t)4 * nb * sizeof(long long),
                                 h->s));
    }
    h->P.bandq = reinterpret_cast<long long *>(h->band + (size_t)12 * nb);
    h->P.band_on = 1;
    h->P.bsx = bs[0];
    h->P.bsy = bs[1];
    h->P.bsz = bs[2];
    h->P.nb = nb;
    // near box: the band grown by the one-cell pull stencil
    {
        // (and to whole row segments of the multi-cell kernel)
        int tx = h->tile_x;
        if (h->vcells > 1 && tx % h->vcells != 0) tx = tx * h->vcells / std::gcd(tx, h->vcells);
        const int tile[3] = {tx, h->tile_y, 1};
        for (int a = 0; a < 3; a++) {
            int lo = std::max(0, org[a] - 1), hi = std::min(dims[a], org[a] + bs[a] + 1);
            lo = (lo / tile[a]) * tile[a];
            hi = std::min(dims[a], ((hi + tile[a] - 1) / tile[a]) * tile[a]);
            h->P.nlo[a] = lo;
            h->P.nhi[a] = hi;
        }
    }
    std::vector<float> ud((size_t)3 * n);
    for (int a = 0; a < 3; a++)
        for (int m = 0; m < n; m++) ud[(size_t)a * n + m] = (float)(udes ? udes[(size_t)a * n + m] : ic->velocity[a]);
    CUDA_TRY(cudaMemcpyAsync(h->mk.pos, xyz, (size_t)3 * n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemcpyAsync(h->mk.ds, ds, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemcpyAsync(h->mk.udes, ud.data(), ud.size() * sizeof(float), cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemsetAsync(h->mk.acc, 0, (size_t)11 * n * sizeof(double), h->s));
    // device state: band origin and rigid body
    DevState d;
    CUDA_TRY(cudaMemcpyAsync(&d, h->ds, sizeof(d), cudaMemcpyDeviceToHost, h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    for (int a = 0; a < 3; a++) {
        d.band_o[a] = org[a];
        d.body_xc[a] = ic->center[a];
        d.body_v[a] = ic->velocity[a];
        d.body_om[a] = 0.0;
        d.body_dxc[a] = 0.0;
    }
    d.have_prev = 0;
    for (int k = 0; k < 6; k++) d.internal_prev[k] = 0.0;
    for (int a = 0; a < 3; a++) d.body_v_prev[a] = d.body_om_prev[a] = 0.0;
    CUDA_TRY(cudaMemcpyAsync(h->ds, &d, sizeof(d), cudaMemcpyHostToDevice, h->s));
    h->bp.free_body = ic->free_body;
    h->bp.radius = ic->radius;
    h->bp.mass = ic->density_ratio * ic->volume;
    h->bp.inertia = ic->inertia;
    for (int a = 0; a < 3; a++)
        h->bp.gacc[a] = ic->density_ratio > 0 ? (1.0 - 1.0 / ic->density_ratio) * ic->gravity[a] : 0.0;
    h->bp.dof = ic->free_dofs ? ic->free_dofs : 63;
    h->bp.vol = ic->volume;
    for (int a = 0; a < 3; a++) h->bp.grav[a] = ic->gravity[a];
    h->bp.mv = ic->virtual_mass * ic->volume;
    h->bp.iv = ic->density_ratio > 0 ? ic->virtual_mass * ic->inertia / ic->density_ratio : 0.0;
    // Keep the band in L2 while the far-region streaming (hundreds of MB)
    // passes through it: a persisting access-policy window on the streams
    // that run the IBM phase.  A per-context limit; best effort.
    {
        int dev = 0, max_persist = 0, max_win = 0;
        if (cudaGetDevice(&dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, dev) == cudaSuccess &&
            cudaDeviceGetAttribute(&max_win, cudaDevAttrMaxAccessPolicyWindowSize, dev) == cudaSuccess &&
            max_persist > 0 && max_win > 0) {
            const size_t bytes =
                std::min<size_t>((size_t)12 * nb * sizeof(float) + (size_t)4 * nb * sizeof(long long), (size_t)max_win);
            size_t cur = 0;
            cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
            if (cur < bytes) cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::min<size_t>(bytes, max_persist));
            cudaStreamAttrValue v;
            memset(&v, 0, sizeof(v));
            v.accessPolicyWindow.base_ptr = h->band;
            v.accessPolicyWindow.num_bytes = bytes;
            v.accessPolicyWindow.hitRatio = 1.0f;
            v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
            v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
            for (cudaStream_t st : {h->s, h->s2, h->s3})
                if (st) cudaStreamSetAttribute(st, cudaStreamAttributeAccessPolicyWindow, &v);
        }
        cudaGetLastError();
    }
    h->ibm = true;
    // graphs captured earlier do not contain the IBM launches
    for (int i = 0; i < 2; i++)
        if (h->gexec[i]) {
            cudaGraphExecDestroy(h->gexec[i]);
            h->gexec[i] = nullptr;
        }
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

// New positions and weights for the markers of the current body (a motion
// prescribed by the caller, the per-step input of IBLBM's marker array):
// copies enqueued on the handle's stream ahead of the next step, nothing
// else reset, captured graphs stay valid (they read the same device arrays).
extern "C" lbm_status lbmgpu_update_markers(lbm_handle *h, const double *xyz, const double *ds) {
    if (!h || !xyz || !ds) return fail(LBM_ERR_INVALID, "update_markers: null argument");
    if (h->d2) return fail(LBM_ERR_UNSUPPORTED, "update_markers: D2Q9 bodies move by their prescribed motion");
    if (!h->ibm) return fail(LBM_ERR_STATE, "update_markers: call lbmgpu_set_markers first");
    const int n = h->mk.n;
    CUDA_TRY(cudaMemcpyAsync(h->mk.pos, xyz, (size_t)3 * n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemcpyAsync(h->mk.ds, ds, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, h->s));
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// Stepping
// ---------------------------------------------------------------------------
static LaunchArgs make_args(lbm_handle *h, int gather) {
    LaunchArgs a;
    a.P = &h->P;
    a.A = h->f[h->cur];
    a.B = h->f[1 - h->cur];
    a.GA = h->g[h->cur];
    a.GB = h->g[1 - h->cur];
    a.ds = h->ds;
    a.mom = nullptr;
    a.band = h->band;
    a.gather = gather;
    a.export_only = 0;
    a.region = 0;
    a.thermal = h->cfg.thermal;
    a.tx = h->tx;
    a.ty = h->ty;
    a.stream = h->s;
    a.vcells = h->solids ? 0 : h->vcells;
    return a;
}

// The IBM phase on stream s.  split: the force reduction (which needs only the
// last interpolation) runs on s3 beside the last spreading and the band
// collision, and the next phase's first interpolation waits for it.
static cudaError_t enqueue_ibm(lbm_handle *h, const LaunchArgs &a, cudaStream_t s, bool split) {
    cudaError_t e;
    IbmArgs ia;
    ia.P = &h->P;
    ia.mk = h->mk;
    ia.ds = h->ds;
    ia.band = h->band;
    ia.thermal = h->icfg.thermal;
    ia.stream = s;
    ia.pdl = h->cfg.storage == LBM_STORE_F32 ? 1 : 0;
    LaunchArgs b = a;
    b.stream = s;
    b.pdl = ia.pdl;
    const float fsign = h->icfg.literal_sign ? -1.0f : 1.0f;
    if (split && (e = cudaStreamWaitEvent(s, h->ev_fin, 0)) != cudaSuccess) return e;
    for (int it = 1; it <= h->icfg.m_max; it++) {
        if ((e = launch_ibm_interp(ia, it == 1 ? 1 : 0, it == h->icfg.m_max ? 1 : 0)) != cudaSuccess) return e;
        if (split && it == h->icfg.m_max) {
            if ((e = cudaEventRecord(h->ev_acc, s)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(h->s3, h->ev_acc, 0)) != cudaSuccess) return e;
            IbmArgs fa = ia;
            fa.stream = h->s3;
            if ((e = launch_ibm_finish(fa, h->bp, h->hist, h->hist_cap)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(h->ev_fin, h->s3)) != cudaSuccess) return e;
        }
        if ((e = launch_ibm_spread(ia)) != cudaSuccess) return e;
    }
    if ((e = launch_band_collide(h->cfg.storage, b, fsign)) != cudaSuccess) return e;
    if (split) return cudaSuccess;
    return launch_ibm_finish(ia, h->bp, h->hist, h->hist_cap);
}

// Enqueue one reference iteration.  ev (optional, 4 events) bracket the fused
// collide-stream launches: ev[0..1] the whole grid or its far region, ev[2..3]
// the near box (recorded as an empty interval when there is none).
//
// With a fixed immersed body the IBM phase of step t runs on a second stream
// while the main stream already streams the cells of step t+1 that do not
// touch the band (the "far" region); only the near box -- the band grown by
// the one-cell pull stencil -- waits for it:
//   main: far(t) | wait ibm(t-1) | near(t) | record near(t)
//   side: wait near(t) | interp/spread x m_max, band collide, finish | record ibm(t)
// A moving body changes the band each step, so it keeps the serial order.
static cudaError_t enqueue_step(lbm_handle *h, int gather, const cudaEvent_t *ev) {
    LaunchArgs a = make_args(h, gather);
    cudaError_t e;
    const bool overlap = h->ibm && gather && !h->icfg.free_body && h->s2 && h->cfg.ibm_overlap >= 0 && !h->solids;
    if (ev) cudaEventRecord(ev[0], h->s);
    if (!overlap) {
        if ((e = launch_step(h->cfg.storage, a)) != cudaSuccess) return e;
        if (h->solids && gather &&
            (e = launch_mea_finish(h->mea_part, h->mea_blocks, h->n_mea_blocks, h->mea_ring, h->mea_cap, h->ds, 1,
                                   h->s)) != cudaSuccess)
            return e;
        if (ev) {
            cudaEventRecord(ev[1], h->s);
            cudaEventRecord(ev[2], h->s);
            cudaEventRecord(ev[3], h->s);
        }
        if (ev) cudaEventRecord(ev[4], h->s);
        if (h->ibm && (e = enqueue_ibm(h, a, h->s, false)) != cudaSuccess) return e;
        if (ev) cudaEventRecord(ev[5], h->s);
        if (h->ibm) cudaEventRecord(h->ev_ibm, h->s);
        h->cur = 1 - h->cur;
        return cudaSuccess;
    }
    a.region = 1;
    if ((e = launch_step(h->cfg.storage, a)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[1], h->s);
    if ((e = cudaStreamWaitEvent(h->s, h->ev_ibm, 0)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[2], h->s);
    a.region = 2;
    if ((e = launch_step(h->cfg.storage, a)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[3], h->s);
    if ((e = cudaEventRecord(h->ev_near, h->s)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(h->s2, h->ev_near, 0)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[4], h->s2);
    if ((e = enqueue_ibm(h, a, h->s2, true)) != cudaSuccess) return e;
    if (ev) cudaEventRecord(ev[5], h->s2);
    if ((e = cudaEventRecord(h->ev_ibm, h->s2)) != cudaSuccess) return e;
    h->cur = 1 - h->cur;
    return cudaSuccess;
}

// Order everything after the last IBM phase on the main stream.
static cudaError_t join_ibm(lbm_handle *h) {
    if (!h->ibm || !h->s2) return cudaSuccess;
    cudaError_t e = cudaStreamWaitEvent(h->s, h->ev_ibm, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(h->s, h->ev_fin, 0);
    return e;
}

static lbm_status ensure_graph(lbm_handle *h) {
    const int p = h->cur;
    if (h->gexec[p]) return LBM_OK;
    cudaGraph_t g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(h->s, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < h->gsteps && e == cudaSuccess; i++) e = enqueue_step(h, 1, nullptr);
    if (e == cudaSuccess) e = join_ibm(h);
    cudaError_t e2 = cudaStreamEndCapture(h->s, &g);
    h->cur = p;  // gsteps is even: the capture ends where it started
    if (e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(LBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    if (e2 != cudaSuccess) return fail(LBM_ERR_CUDA, std::string("graph capture end: ") + cudaGetErrorString(e2));
    cudaError_t e3 = cudaGraphInstantiate(&h->gexec[p], g, 0);
    cudaGraphDestroy(g);
    if (e3 != cudaSuccess) {
        h->gexec[p] = nullptr;
        return fail(LBM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e3));
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_step(lbm_handle *h, int nsteps) {
    if (!h) return fail(LBM_ERR_INVALID, "step: null handle");
    if (h->d2) return l2d_step(h, nsteps);
    if (!h->inited) return fail(LBM_ERR_STATE, "step: call lbmgpu_init first");
    if (nsteps < 0) return fail(LBM_ERR_INVALID, "step: negative step count");
    while (nsteps > 0) {
        if (h->steps == 0) {
            CUDA_TRY(enqueue_step(h, 0, nullptr));
            h->steps++;
            nsteps--;
            continue;
        }
        if (h->gsteps > 0 && nsteps >= h->gsteps) {
            if (ensure_graph(h) != LBM_OK) {
                // a launch that cannot be captured on this device/driver:
                // keep stepping eagerly from now on
                cudaGetLastError();
                h->gsteps = 0;
                continue;
            }
            CUDA_TRY(cudaGraphLaunch(h->gexec[h->cur], h->s));
            // the graph ends joined on the main stream; re-arm the IBM event
            // outside the capture so later waits on it are ordinary ones
            if (h->ibm && h->s2) {
                CUDA_TRY(cudaEventRecord(h->ev_ibm, h->s));
                CUDA_TRY(cudaEventRecord(h->ev_fin, h->s));
            }
            h->steps += h->gsteps;
            nsteps -= h->gsteps;
            continue;
        }
        CUDA_TRY(enqueue_step(h, 1, nullptr));
        h->steps++;
        nsteps--;
    }
    CUDA_TRY(join_ibm(h));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_step_timed(lbm_handle *h, int nsteps, double *ms) {
    if (!h || !ms) return fail(LBM_ERR_INVALID, "step_timed: null argument");
    CUDA_TRY(cudaEventRecord(h->ev[0], h->s));
    lbm_status st = lbmgpu_step(h, nsteps);
    if (st != LBM_OK) return st;
    CUDA_TRY(cudaEventRecord(h->ev[1], h->s));
    CUDA_TRY(cudaEventSynchronize(h->ev[1]));
    float t = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&t, h->ev[0], h->ev[1]));
    *ms = t;
    return LBM_OK;
}

// Steps launched one by one with six events each: far/whole fused launch,
// near launch, IBM phase (on whichever stream runs it).
static lbm_status step_phases(lbm_handle *h, int nsteps, double *total, double *fused, double *near_ms,
                              double *ibm_ms) {
    if (!h) return fail(LBM_ERR_INVALID, "step_profiled: null handle");
    if (h->d2) return fail(LBM_ERR_UNSUPPORTED, "step_profiled: not for D2Q9 handles (use lbmgpu_step_timed)");
    if (!h->inited) return fail(LBM_ERR_STATE, "step_profiled: call lbmgpu_init first");
    if (nsteps < 0) return fail(LBM_ERR_INVALID, "step_profiled: negative step count");
    // all events are read after the last step so the host never stalls the
    // stream between steps
    while ((int)h->evpool.size() < 6 * nsteps) {
        cudaEvent_t e;
        CUDA_TRY(cudaEventCreate(&e));
        h->evpool.push_back(e);
    }
    CUDA_TRY(cudaEventRecord(h->ev[0], h->s));
    for (int i = 0; i < nsteps; i++) {
        CUDA_TRY(enqueue_step(h, h->steps == 0 ? 0 : 1, &h->evpool[6 * i]));
        h->steps++;
    }
    CUDA_TRY(join_ibm(h));
    CUDA_TRY(cudaEventRecord(h->ev[1], h->s));
    CUDA_TRY(cudaEventSynchronize(h->ev[1]));
    float tot = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&tot, h->ev[0], h->ev[1]));
    double far = 0.0, nr = 0.0, ib = 0.0;
    for (int i = 0; i < nsteps; i++) {
        const cudaEvent_t *e = &h->evpool[6 * i];
        float a = 0.f, b = 0.f, c = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&a, e[0], e[1]));
        CUDA_TRY(cudaEventElapsedTime(&b, e[2], e[3]));
        CUDA_TRY(cudaEventElapsedTime(&c, e[4], e[5]));
        far += a;
        nr += b;
        ib += c;
    }
    if (total) *total = tot;
    if (fused) *fused = far + nr;
    if (near_ms) *near_ms = nr;
    if (ibm_ms) *ibm_ms = ib;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_step_profiled(lbm_handle *h, int nsteps, double *total_ms, double *fused_ms) {
    return step_phases(h, nsteps, total_ms, fused_ms, nullptr, nullptr);
}

extern "C" lbm_status lbmgpu_step_phases(lbm_handle *h, int nsteps, double *phases) {
    if (!phases) return fail(LBM_ERR_INVALID, "step_phases: null argument");
    return step_phases(h, nsteps, &phases[0], &phases[1], &phases[2], &phases[3]);
}

// ---------------------------------------------------------------------------
// Read-back
// ---------------------------------------------------------------------------
// Gather-only pass writing the moments of the current state into h->mom,
// after any asynchronous output copy of the previous contents.
cudaError_t lbm_export_moments_async(lbm_handle *h) {
    cudaError_t e = lbm_mom_acquire(h);
    if (e != cudaSuccess) return e;
    LaunchArgs a = make_args(h, h->steps == 0 ? 0 : 1);
    a.mom = h->mom;
    a.export_only = 1;
    return launch_step(h->cfg.storage, a);
}

static lbm_status export_moments(lbm_handle *h) {
    if (!h->inited) return fail(LBM_ERR_STATE, "download: call lbmgpu_init first");
    CUDA_TRY(lbm_export_moments_async(h));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download_f32(lbm_handle *h, int field, float *host) {
    if (!h || !host) return fail(LBM_ERR_INVALID, "download: null argument");
    if (h->d2) return l2d_download_f32(h, field, host);
    if (field < 0 || field > 7 || (field >= 4 && !h->cfg.thermal)) return fail(LBM_ERR_INVALID, "download: bad field");
    lbm_status s = export_moments(h);
    if (s != LBM_OK) return s;
    CUDA_TRY(cudaMemcpyAsync(host, h->mom + (size_t)field * h->P.N, (size_t)h->P.N * sizeof(float),
                             cudaMemcpyDeviceToHost, h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download_all_f32(lbm_handle *h, float *host) {
    if (!h || !host) return fail(LBM_ERR_INVALID, "download: null argument");
    if (h->d2) return l2d_download_all_f32(h, host);
    lbm_status s = export_moments(h);
    if (s != LBM_OK) return s;
    const int nf = h->cfg.thermal ? 5 : 4;
    CUDA_TRY(cudaMemcpyAsync(host, h->mom, (size_t)nf * h->P.N * sizeof(float), cudaMemcpyDeviceToHost, h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

// The device address of pinned, device-mapped host memory (lbmgpu_host_alloc),
// else null.
static const void *mapped_device_ptr(const void *host) {
    cudaPointerAttributes pa;
    const void *d = nullptr;
    if (cudaPointerGetAttributes(&pa, host) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
        d = pa.devicePointer;
    cudaGetLastError();
    return d;
}

// Device-to-host copy done by a few blocks that store straight into pinned,
// device-mapped host memory.  A copy-engine transfer of the moments (tens of
// MB) would sit in front of every small read-back the caller makes meanwhile
// (force rows, status words); these stores leave the copy engines free and
// run beside the next steps.  16 blocks reach the same host-link rate as 64
// (67 MB in about 0.38 ms on a GB300); fewer take fewer SM slots from the
// steps they overlap, until the copy no longer ends within them.  Measured
// end to end on the FP16 sphere channel (10 steps per call): 4 blocks 31.1 k,
// 6 36.1 k, 8 36.2 k, 10 36.5 k, 12 35.2 k, 16 34.2 k MLUPS.
__global__ void __launch_bounds__(512) k_copy_out(const float *__restrict__ src, float *__restrict__ dst, long long n) {
    const long long n4 = n >> 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const float4 *s4 = reinterpret_cast<const float4 *>(src);
    float4 *d4 = reinterpret_cast<float4 *>(dst);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += stride) d4[i] = __ldcs(s4 + i);
    for (long long i = (n4 << 2) + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

extern "C" lbm_status lbmgpu_download_all_f32_async(lbm_handle *h, float *host) {
    if (!h || !host) return fail(LBM_ERR_INVALID, "download: null argument");
    if (h->d2) return l2d_download_all_f32(h, host);  // synchronous on D2Q9 handles
    if (!h->s_dl) {
        CUDA_TRY(cudaStreamCreateWithFlags(&h->s_dl, cudaStreamNonBlocking));
        CUDA_TRY(cudaEventCreateWithFlags(&h->ev_dl_exported, cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&h->ev_dl_copied, cudaEventDisableTiming));
    }
    // the export waits for the previous copy out of h->mom (lbm_mom_acquire)
    lbm_status s = export_moments(h);
    if (s != LBM_OK) return s;
    const int nf = h->cfg.thermal ? 5 : 4;
    CUDA_TRY(cudaEventRecord(h->ev_dl_exported, h->s));
    CUDA_TRY(cudaStreamWaitEvent(h->s_dl, h->ev_dl_exported, 0));
    const long long n = (long long)nf * h->P.N;
    // pinned memory the device can address (lbmgpu_host_alloc): stored by a
    // kernel; anything else: a copy-engine transfer
    void *dptr = const_cast<void *>(mapped_device_ptr(host));
    if (((uintptr_t)dptr & 15u) != 0) dptr = nullptr;
    if (dptr) {
        k_copy_out<<<10, 512, 0, h->s_dl>>>(h->mom, (float *)dptr, n);
        CUDA_TRY(cudaGetLastError());
    } else {
        CUDA_TRY(cudaMemcpyAsync(host, h->mom, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, h->s_dl));
    }
    CUDA_TRY(cudaEventRecord(h->ev_dl_copied, h->s_dl));
    h->dl_issued = true;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download_wait(lbm_handle *h) {
    if (!h) return fail(LBM_ERR_INVALID, "download_wait: null handle");
    if (h->s_dl) CUDA_TRY(cudaStreamSynchronize(h->s_dl));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_download(lbm_handle *h, int field, double *host) {
    if (!h || !host) return fail(LBM_ERR_INVALID, "download: null argument");
    std::vector<float> tmp((size_t)h->cfg.nx * h->cfg.ny * h->cfg.nz);
    lbm_status s = lbmgpu_download_f32(h, field, tmp.data());
    if (s != LBM_OK) return s;
    for (size_t i = 0; i < tmp.size(); i++) host[i] = tmp[i];
    return LBM_OK;
}

// ---------------------------------------------------------------------------
// Interior solid cells (staircase bodies) and their momentum exchange
// ---------------------------------------------------------------------------
extern "C" lbm_status lbmgpu_set_solids(lbm_handle *h, const uint8_t *mask) {
    if (!h || !mask) return fail(LBM_ERR_INVALID, "set_solids: null argument");
    if (h->d2) return l2d_set_solids(h, mask);
    if (h->inited) return fail(LBM_ERR_STATE, "set_solids: call before lbmgpu_init");
    if (h->solids) return fail(LBM_ERR_STATE, "set_solids: solids already set");
    const int nx = h->P.nx, ny = h->P.ny, nz = h->P.nz;
    const long long N = h->P.N, words = (N + 31) / 32;
    std::vector<uint32_t> sol((size_t)words, 0u), nea((size_t)words, 0u);
    long long nsolid = 0;
    for (long long c = 0; c < N; c++)
        if (mask[c]) {
            sol[(size_t)(c >> 5)] |= 1u << (c & 31);
            nsolid++;
        }
    if (nsolid == 0) return fail(LBM_ERR_INVALID, "set_solids: no solid cell");
    // near: a solid, or a cell one of whose 18 neighbours is one
    const int per = h->P.periodic;
    const int gx = (nx + h->tx - 1) / h->tx, gy = (ny + h->ty - 1) / h->ty;
    std::vector<char> blk((size_t)gx * gy * nz, 0);
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const long long c = x + (long long)nx * (y + (long long)ny * z);
                bool nr = mask[c] != 0;
                for (int l = 1; l < Q && !nr; l++) {
                    int sx = x - cx(l), sy = y - cy(l), sz = z - cz(l);
                    if (per & 1) sx = (sx + nx) % nx;
                    if (per & 2) sy = (sy + ny) % ny;
                    if (per & 4) sz = (sz + nz) % nz;
                    if (sx < 0 || sy < 0 || sz < 0 || sx >= nx || sy >= ny || sz >= nz) continue;
                    nr = mask[sx + (long long)nx * (sy + (long long)ny * sz)] != 0;
                }
                if (nr) {
                    nea[(size_t)(c >> 5)] |= 1u << (c & 31);
                    blk[(size_t)(x / h->tx) + (size_t)gx * ((size_t)(y / h->ty) + (size_t)gy * z)] = 1;
                }
            }
    std::vector<int> list;
    for (size_t b = 0; b < blk.size(); b++)
        if (blk[b]) list.push_back((int)b);
    CUDA_TRY(dalloc(h, &h->solid_d, (size_t)words * 4));
    CUDA_TRY(dalloc(h, &h->near_d, (size_t)words * 4));
    CUDA_TRY(dalloc(h, &h->mea_part, blk.size() * 3 * sizeof(float)));
    CUDA_TRY(dalloc(h, &h->mea_blocks, list.size() * sizeof(int)));
    CUDA_TRY(dalloc(h, &h->mea_ring, (size_t)h->mea_cap * 4 * sizeof(double)));
    CUDA_TRY(cudaMemcpyAsync(h->solid_d, sol.data(), (size_t)words * 4, cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemcpyAsync(h->near_d, nea.data(), (size_t)words * 4, cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemcpyAsync(h->mea_blocks, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, h->s));
    CUDA_TRY(cudaMemsetAsync(h->mea_part, 0, blk.size() * 3 * sizeof(float), h->s));
    CUDA_TRY(cudaMemsetAsync(h->mea_ring, 0, (size_t)h->mea_cap * 4 * sizeof(double), h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    h->n_mea_blocks = (int)list.size();
    h->P.solid = h->solid_d;
    h->P.nearw = h->near_d;
    h->P.mea = h->mea_part;
    h->solids = true;
    for (int i = 0; i < 2; i++)
        if (h->gexec[i]) {
            cudaGraphExecDestroy(h->gexec[i]);
            h->gexec[i] = nullptr;
        }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_mea_box(lbm_handle *h, const int box[6], double out[3]) {
    if (!h || !box || !out) return fail(LBM_ERR_INVALID, "mea_box: null argument");
    if (!h->d2)
        return fail(LBM_ERR_UNSUPPORTED, "mea_box: D2Q9 handles; a D3Q19 handle sums every solid (get_solid_forces)");
    return l2d_mea_box(h, box, out);
}

extern "C" lbm_status lbmgpu_get_solid_forces(lbm_handle *h, double *out, int max_steps, int *n_out) {
    if (!h || !out || max_steps < 0) return fail(LBM_ERR_INVALID, "get_solid_forces: bad argument");
    if (h->d2) return fail(LBM_ERR_UNSUPPORTED, "get_solid_forces: D2Q9 handles take lbmgpu_mea_box");
    if (!h->solids) return fail(LBM_ERR_STATE, "get_solid_forces: no solid cells set");
    if (!h->inited) return fail(LBM_ERR_STATE, "get_solid_forces: call lbmgpu_init first");
    long long n = 0;
    if (h->steps >= 1) {
        // the latest step's exchange needs its streamed populations: one
        // gather-only pass, recorded without advancing (the next step
        // recomputes the same record)
        LaunchArgs a = make_args(h, 1);
        a.export_only = 1;
        CUDA_TRY(launch_step(h->cfg.storage, a));
        CUDA_TRY(launch_mea_finish(h->mea_part, h->mea_blocks, h->n_mea_blocks, h->mea_ring, h->mea_cap, h->ds, 0,
                                   h->s));
        // records of reference steps 1 .. steps
        n = std::min<long long>(std::min<long long>(h->steps, h->mea_cap), max_steps);
        const long long last = h->steps;
        long long first = (last - n + 1) % h->mea_cap;
        long long n1 = std::min(n, h->mea_cap - first);
        if (n1 > 0)
            CUDA_TRY(cudaMemcpyAsync(out, h->mea_ring + first * 4, (size_t)n1 * 4 * sizeof(double),
                                     cudaMemcpyDeviceToHost, h->s));
        if (n > n1)
            CUDA_TRY(cudaMemcpyAsync(out + n1 * 4, h->mea_ring, (size_t)(n - n1) * 4 * sizeof(double),
                                     cudaMemcpyDeviceToHost, h->s));
        CUDA_TRY(cudaStreamSynchronize(h->s));
    }
    if (n_out) *n_out = (int)n;
    return LBM_OK;
}

// The last n = min(steps done, ring size, rows) rows of the force ring, in
// step order, and n after them, stored into pinned, device-mapped host memory.
// The device knows the step count, so the read-back is one launch and one
// synchronisation, and it takes no copy engine (a moments download may hold
// one for a few hundred microseconds).
__global__ void k_forces_out(const DevState *__restrict__ ds, const double *__restrict__ hist, long long cap,
                             long long rows, double *__restrict__ dst) {
    const long long step = ds->step;
    const long long n = min(min(step, cap), rows);
    const long long first = step - n;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n * 8;
         e += (long long)gridDim.x * blockDim.x)
        dst[e] = hist[((first + (e >> 3)) % cap) * 8 + (e & 7)];
    if (blockIdx.x == 0 && threadIdx.x == 0) dst[rows * 8] = (double)n;
}

extern "C" lbm_status lbmgpu_get_forces(lbm_handle *h, double *out, int max_steps, int *n_out) {
    if (!h || !out || max_steps < 0) return fail(LBM_ERR_INVALID, "get_forces: bad argument");
    if (h->d2) return l2d_get_forces(h, out, max_steps, n_out);
    if (!h->ibm) return fail(LBM_ERR_STATE, "get_forces: no markers set");
    const long long rows = std::min<long long>(max_steps, h->hist_cap);
    if (rows > h->fstage_rows || !h->fstage) {
        if (h->fstage) {
            CUDA_TRY(cudaStreamSynchronize(h->s));
            CUDA_TRY(cudaFreeHost(h->fstage));
            h->fstage = nullptr;
            h->fstage_rows = 0;
        }
        const long long cap = std::max<long long>(rows, 64);
        CUDA_TRY(cudaHostAlloc((void **)&h->fstage, (size_t)(cap * 8 + 1) * sizeof(double), cudaHostAllocMapped));
        h->fstage_rows = cap;
    }
    double *dst = nullptr;
    CUDA_TRY(cudaHostGetDevicePointer((void **)&dst, h->fstage, 0));
    const unsigned blocks = (unsigned)std::min<long long>((rows * 8 + 255) / 256 + 1, 64);
    k_forces_out<<<blocks, 256, 0, h->s>>>(h->ds, h->hist, h->hist_cap, rows, dst);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->s));
    const long long n = (long long)h->fstage[rows * 8];
    std::memcpy(out, h->fstage, (size_t)n * 8 * sizeof(double));
    if (n_out) *n_out = (int)n;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_set_marker_normals(lbm_handle *h, const double *nxyz) {
    if (!h || !nxyz) return fail(LBM_ERR_INVALID, "set_marker_normals: null argument");
    if (!h->d2) return fail(LBM_ERR_UNSUPPORTED, "set_marker_normals: D2Q9 handles only");
    return l2d_set_normals(h, nxyz);
}

extern "C" lbm_status lbmgpu_get_body(lbm_handle *h, double out[9]) {
    if (!h || !out) return fail(LBM_ERR_INVALID, "get_body: null argument");
    if (h->d2) return l2d_get_body(h, out);
    DevState d;
    CUDA_TRY(cudaMemcpyAsync(&d, h->ds, sizeof(d), cudaMemcpyDeviceToHost, h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    for (int a = 0; a < 3; a++) {
        out[a] = d.body_xc[a];
        out[3 + a] = d.body_v[a];
        out[6 + a] = d.body_om[a];
    }
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_get_markers(lbm_handle *h, double *xyz) {
    if (!h || !xyz) return fail(LBM_ERR_INVALID, "get_markers: null argument");
    if (h->d2) return l2d_get_markers(h, xyz);
    if (!h->ibm) return fail(LBM_ERR_STATE, "get_markers: no markers set");
    CUDA_TRY(cudaMemcpyAsync(xyz, h->mk.pos, (size_t)3 * h->mk.n * sizeof(double), cudaMemcpyDeviceToHost, h->s));
    CUDA_TRY(cudaStreamSynchronize(h->s));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_status(lbm_handle *h, uint32_t *flags) {
    if (!h || !flags) return fail(LBM_ERR_INVALID, "status: null argument");
    uint32_t v = 0;
    if (h->d2) {
        lbm_status st = l2d_status(h, &v);
        if (st != LBM_OK) return st;
    } else {
        CUDA_TRY(cudaMemcpyAsync(&v, &h->ds->status, sizeof(v), cudaMemcpyDeviceToHost, h->s));
        CUDA_TRY(cudaStreamSynchronize(h->s));
    }
    *flags = v;
    if (v & ST_RHO_RANGE) return fail(LBM_ERR_DIVERGED, "status: density left (0, 100) or became NaN");
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_sync(lbm_handle *h) {
    if (!h) return fail(LBM_ERR_INVALID, "sync: null handle");
    CUDA_TRY(cudaStreamSynchronize(h->s));
    if (h->s_dl) CUDA_TRY(cudaStreamSynchronize(h->s_dl));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_steps_done(lbm_handle *h, long long *steps) {
    if (!h || !steps) return fail(LBM_ERR_INVALID, "steps_done: null argument");
    *steps = h->steps;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_device_bytes(lbm_handle *h, size_t *bytes) {
    if (!h || !bytes) return fail(LBM_ERR_INVALID, "device_bytes: null argument");
    *bytes = h->dev_bytes;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_cells_per_thread(lbm_handle *h, int *cells) {
    if (!h || !cells) return fail(LBM_ERR_INVALID, "cells_per_thread: null argument");
    *cells = (h->d2 || h->solids || h->vcells <= 1) ? 1 : h->vcells;
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return fail(LBM_ERR_INVALID, "host_alloc: null argument");
    CUDA_TRY(cudaMallocHost(ptr, bytes));
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_host_free(void *ptr) {
    CUDA_TRY(cudaFreeHost(ptr));
    return LBM_OK;
}
