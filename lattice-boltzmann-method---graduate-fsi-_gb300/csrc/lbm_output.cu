// lbm_output.cu -- output of the solver state in the reference's file formats,
// written by a host thread while the device keeps stepping.
//
//   lbmgpu_output_vtk_async   OutputVTK (lbm.cpp:2290-2642): RectilinearGrid,
//                             appended raw Float32 cell data
//   lbmgpu_output_markers_vtk OutputVTK_Marker (lbm.cpp:3033-3077): legacy
//                             ASCII POLYDATA of the markers
//   lbmgpu_output_csv         OutputCSV (lbm.cpp:3169-3186): "time,error"
//
// The VTK path: a gather-only export pass writes the moments into the
// handle's moment buffer on the main stream; a copy stream moves them to
// pinned host memory once that pass is done; a writer thread waits for the
// copy and formats the file.  The main stream goes on with the next steps
// meanwhile -- only the next writer of the moment buffer (download, init
// from fields, the next output) waits for the copy.  One file is in flight at
// a time: a new call first finishes the previous one.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

#include "lbm_handle.h"

struct lbm_output {
    float *host = nullptr;  // pinned: moments, then the band snapshot
    size_t host_floats = 0;
    cudaStream_t copy = nullptr;
    cudaEvent_t exported = nullptr, copied = nullptr;
    bool copy_issued = false;
    std::thread writer;
    lbm_status result = LBM_OK;  // of the last finished write
    std::string error;
};

namespace {

lbm_status out_fail(lbm_status s, const std::string &m) {
    lbm_set_last_error(m);
    return s;
}

// Wait for the writer in flight; its status becomes the call's.
lbm_status join_writer(lbm_output *o) {
    if (o->writer.joinable()) o->writer.join();
    lbm_status r = o->result;
    if (r != LBM_OK) lbm_set_last_error(o->error);
    o->result = LBM_OK;
    return r;
}

// Reference cell-type code of a face kind (LBM.h:505-515).
float face_type(int kind) {
    switch (kind) {
    case LBM_FACE_WALL: return 1.0f;                                  // TYPE_S
    case LBM_FACE_INLET: return 3.0f;                                 // TYPE_IN
    case LBM_FACE_OUTLET_EQ: case LBM_FACE_OUTLET_ZG: return 2.0f;    // TYPE_OUT
    default: return 0.0f;                                             // TYPE_F
    }
}

// Cells of a reference-layout file: i = 0..Nx+1, j = 0..Ny+1, k = 1..Nz of
// the reference's fluid array, ghosts included.
struct VtkGrid {
    lbm_config cfg;
    int dn[3];      // device extent
    int nref[3];    // reference interior extent (N, or device - 2 on a periodic axis)
    int off[3];     // device cell = reference index - off
    long long N;
    std::vector<uint8_t> types;  // ghost-inclusive cell types given by the caller, or empty
    std::vector<uint32_t> solid; // packed interior solid mask (device extent), or empty

    // device cell of reference cell (i, j, k), or -1 for a ghost (side[] set)
    long long locate(int i, int jj, int k, int side[3]) const {
        const int r[3] = {i, jj, k};
        long long d[3];
        bool ghost = false;
        for (int a = 0; a < 3; a++) {
            side[a] = -1;
            const int v = r[a] - off[a];
            if (v < 0) {
                side[a] = 0;
                ghost = true;
            } else if (v >= dn[a]) {
                side[a] = 1;
                ghost = true;
            }
            d[a] = v;
        }
        if (ghost) return -1;
        return d[0] + (long long)dn[0] * (d[1] + (long long)dn[1] * d[2]);
    }
};

// Boundary state of a ghost cell: among the faces that contain it, a moving
// wall first (as the class tables do at edges), else the lowest axis.
const lbm_face *ghost_face(const lbm_config &c, const int side[3]) {
    const lbm_face *pick = nullptr;
    for (int a = 0; a < 3; a++) {
        if (side[a] < 0) continue;
        const lbm_face *f = &c.faces[2 * a + side[a]];
        const bool moving = f->kind == LBM_FACE_WALL && (f->u[0] != 0 || f->u[1] != 0 || f->u[2] != 0);
        if (!pick || moving) pick = f;
        if (moving) break;
    }
    return pick;
}

// One cell-data array: its name, components, and the values of a cell --
// an interior cell c >= 0, or a ghost (c < 0) in the state of face gf.
struct VtkArray {
    const char *name;
    int comps;
    std::function<void(long long c, const lbm_face *gf, float *v)> value;
};

VtkGrid grid_of(lbm_handle *h) {
    VtkGrid g;
    g.cfg = h->cfg;
    g.N = h->P.N;
    for (int a = 0; a < 3; a++) {
        g.dn[a] = a == 0 ? h->P.nx : (a == 1 ? h->P.ny : h->P.nz);
        const bool per = h->cfg.faces[2 * a].kind == LBM_FACE_PERIODIC;
        g.off[a] = per ? 0 : 1;
        g.nref[a] = per ? g.dn[a] - 2 : g.dn[a];
    }
    return g;
}

// The grid of a D2Q9 handle: the computational layer k = 1 of the
// reference's fluid[Nx+2][Ny+2][3], written as one plane.
VtkGrid grid_of_2d(lbm_handle *h) {
    VtkGrid g;
    g.cfg = h->cfg;
    g.N = (long long)h->cfg.nx * h->cfg.ny;
    for (int a = 0; a < 2; a++) {
        g.dn[a] = a == 0 ? h->cfg.nx : h->cfg.ny;
        const bool per = h->cfg.faces[2 * a].kind == LBM_FACE_PERIODIC;
        g.off[a] = per ? 0 : 1;
        g.nref[a] = per ? g.dn[a] - 2 : g.dn[a];
    }
    g.dn[2] = 1;
    g.off[2] = 1;
    g.nref[2] = 1;
    return g;
}

// The caller's types array, else the device solid mask (read on h->s).
bool grid_types(lbm_handle *h, VtkGrid &g, const uint8_t *types) {
    if (types && h->d2) {
        // D2Q9: the caller's (Nx+2)(Ny+2) layer k = 1
        const size_t nt = (size_t)(g.nref[0] + 2) * (g.nref[1] + 2);
        g.types.assign((size_t)(g.nref[0] + 2) * (g.nref[1] + 2) * 3, 0);
        std::copy(types, types + nt, g.types.begin() + nt);
    } else if (types) {
        const size_t nt = (size_t)(g.nref[0] + 2) * (g.nref[1] + 2) * (g.nref[2] + 2);
        g.types.assign(types, types + nt);
    } else if (h->solids) {
        const size_t words = (size_t)((g.N + 31) / 32);
        g.solid.resize(words);
        if (cudaMemcpyAsync(g.solid.data(), h->solid_d, words * 4, cudaMemcpyDeviceToHost, h->s) != cudaSuccess ||
            cudaStreamSynchronize(h->s) != cudaSuccess)
            return false;
    }
    return true;
}

// A RectilinearGrid .vtr in the layout of the reference's writers
// (lbm.cpp:2290-2642, 2644-3031): the arrays, then CellType, cell-vertex
// coordinates, appended raw Float32 data with UInt32 byte counts.
bool write_rectilinear(const std::string &path, const VtkGrid &g, const std::vector<VtkArray> &arrays,
                       std::string &err) {
    const int Nx = g.nref[0], Ny = g.nref[1], Nz = g.nref[2];
    const int zc = Nz;  // planes k = 1 .. Nz, as the reference writes (zcomp)
    const size_t ncell = (size_t)(Nx + 2) * (Ny + 2) * zc;
    FILE *fp = fopen(path.c_str(), "wb");
    if (!fp) {
        err = "cannot open " + path;
        return false;
    }
    unsigned long offset = 0;
    fprintf(fp, "<?xml version=\"1.0\"?>\n");
    fprintf(fp, "<VTKFile type=\"RectilinearGrid\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt32\">\n");
    fprintf(fp, "  <RectilinearGrid WholeExtent=\"0 %d 0 %d 0 %d\">\n", Nx + 2, Ny + 2, zc);
    fprintf(fp, "  <Piece Extent=\"0 %d 0 %d 0 %d\">\n", Nx + 2, Ny + 2, zc);
    fprintf(fp, "    <PointData>\n");
    fprintf(fp, "    </PointData>\n");
    fprintf(fp, "    <CellData>\n");
    auto decl = [&](const char *name, int comps) {
        if (comps == 1)
            fprintf(fp, "      <DataArray type=\"Float32\" Name=\"%s\" format=\"appended\" offset=\"%ld\" />\n", name,
                    (long)offset);
        else
            fprintf(fp,
                    "      <DataArray type=\"Float32\" Name=\"%s\" NumberOfComponents=\"%d\" format=\"appended\" "
                    "offset=\"%ld\" />\n",
                    name, comps, (long)offset);
        offset += 4 + (unsigned long)comps * 4 * ncell;
    };
    for (const VtkArray &a : arrays) decl(a.name, a.comps);
    decl("CellType", 1);
    fprintf(fp, "    </CellData>\n");
    fprintf(fp, "    <Coordinates>\n");
    fprintf(fp, "      <DataArray type=\"Float32\" Name=\"CoordinateX\" format=\"appended\" offset=\"%ld\" />\n",
            (long)offset);
    offset += 4 + 4 * (unsigned long)(Nx + 3);
    fprintf(fp, "      <DataArray type=\"Float32\" Name=\"CoordinateY\" format=\"appended\" offset=\"%ld\" />\n",
            (long)offset);
    offset += 4 + 4 * (unsigned long)(Ny + 3);
    fprintf(fp, "      <DataArray type=\"Float32\" Name=\"CoordinateZ\" format=\"appended\" offset=\"%ld\" />\n",
            (long)offset);
    fprintf(fp, "    </Coordinates>\n");
    fprintf(fp, "  </Piece>\n");
    fprintf(fp, "  </RectilinearGrid>\n");
    fprintf(fp, "  <AppendedData encoding=\"raw\">");
    fprintf(fp, "_");

    const int NXr = Nx + 2, NYr = Ny + 2;
    std::vector<float> buf;
    buf.reserve(9 * ncell);
    auto flush = [&](int comps) {
        const uint32_t bytes = (uint32_t)(comps * 4 * ncell);
        fwrite(&bytes, sizeof(uint32_t), 1, fp);
        fwrite(buf.data(), sizeof(float), buf.size(), fp);
        buf.clear();
    };
    for (const VtkArray &a : arrays) {
        for (int k = 1; k <= zc; k++)
            for (int jj = 0; jj < NYr; jj++)
                for (int i = 0; i < NXr; i++) {
                    int side[3];
                    const long long c = g.locate(i, jj, k, side);
                    float v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                    a.value(c, c >= 0 ? nullptr : ghost_face(g.cfg, side), v);
                    for (int q = 0; q < a.comps; q++) buf.push_back(v[q]);
                }
        flush(a.comps);
    }
    // CellType: the float value of the reference's type code
    for (int k = 1; k <= zc; k++)
        for (int jj = 0; jj < NYr; jj++)
            for (int i = 0; i < NXr; i++) {
                float t;
                if (!g.types.empty()) {
                    t = (float)g.types[(size_t)i + (size_t)NXr * ((size_t)jj + (size_t)NYr * k)];
                } else {
                    int side[3];
                    const long long c = g.locate(i, jj, k, side);
                    if (c >= 0)
                        t = (!g.solid.empty() && ((g.solid[(size_t)(c >> 5)] >> (c & 31)) & 1u)) ? 1.0f : 0.0f;
                    else
                        t = face_type(ghost_face(g.cfg, side)->kind);
                }
                buf.push_back(t);
            }
    flush(1);
    // coordinates of the cell vertices
    for (int a = 0; a < 3; a++) {
        const int n = a == 0 ? Nx + 3 : (a == 1 ? Ny + 3 : zc + 1);
        const uint32_t bytes = (uint32_t)(4 * n);
        fwrite(&bytes, sizeof(uint32_t), 1, fp);
        for (int i = 0; i < n; i++) {
            const float v = (float)i;
            fwrite(&v, sizeof(float), 1, fp);
        }
    }
    fprintf(fp, "  </AppendedData>\n");
    fprintf(fp, "</VTKFile>\n");
    if (fclose(fp) != 0) {
        err = "write failed: " + path;
        return false;
    }
    return true;
}

// sigma (6 distinct components, xx xy xz yy yz zz) as the 9 of a 3x3 tensor
const int kSym9[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};

// MORE_DETAILS arrays of a ghost cell: the face's equilibrium, whose central
// second moment is rho cs^2 delta.
float ghost_pressure(const lbm_face *gf) { return (float)(gf->rho / 3.0); }
float ghost_stress_diag(const lbm_face *gf, double tau) { return (float)(-(tau - 0.5) * (gf->rho / 3.0) / tau); }

struct VtkJob {
    std::string path;
    VtkGrid grid;
    double u_ref, tau;
    int thermal, force, details;
    const float *mom;     // pinned moments
    const float *band;    // pinned band snapshot (force density) or null
    const float *det;     // pinned pressure and stress, or null
    int band_o[3], bs[3];
    float fsign;
    float body[3];
    cudaEvent_t copied;   // null: the host copies are complete (D2Q9)
    // D2Q9 IBM: the force the box cells collided with (rows 0 and 1 of
    // [4][fcap], box order) and the box {x0, y0, w, h}
    int d2 = 0;
    std::vector<float> boxF;
    long long fcap = 0;
    int fbox[4] = {0, 0, 0, 0};
};

void write_vtk(VtkJob j, lbm_output *o) {
    if (j.copied && cudaEventSynchronize(j.copied) != cudaSuccess) {
        o->result = LBM_ERR_CUDA;
        o->error = "output_vtk: copy failed";
        return;
    }
    const long long N = j.grid.N;
    const int *dn = j.grid.dn;
    std::vector<VtkArray> arrays;
    arrays.push_back({"Density", 1, [&](long long c, const lbm_face *gf, float *v) {
                          v[0] = c >= 0 ? j.mom[c] : (float)gf->rho;
                      }});
    arrays.push_back({"Velocity", 3, [&](long long c, const lbm_face *gf, float *v) {
                          for (int a = 0; a < 3; a++)
                              v[a] = c >= 0 ? (float)(j.mom[(1 + a) * N + c] / j.u_ref) : (float)(gf->u[a] / j.u_ref);
                      }});
    if (j.force && j.d2)
        arrays.push_back({"Force density", 3, [&](long long c, const lbm_face *, float *v) {
                              if (c < 0) return;
                              for (int a = 0; a < 3; a++) v[a] = j.body[a];
                              const int bx = (int)(c % dn[0]) - j.fbox[0], by = (int)(c / dn[0]) - j.fbox[1];
                              if ((unsigned)bx < (unsigned)j.fbox[2] && (unsigned)by < (unsigned)j.fbox[3]) {
                                  const long long q = bx + (long long)j.fbox[2] * by;
                                  v[0] = j.boxF[q];
                                  v[1] = j.boxF[j.fcap + q];
                              }
                          }});
    else if (j.force)
        arrays.push_back({"Force density", 3, [&](long long c, const lbm_face *, float *v) {
                              if (c < 0) return;
                              for (int a = 0; a < 3; a++) v[a] = j.body[a];
                              const int bx = (int)(c % dn[0]) - j.band_o[0];
                              const int by = (int)((c / dn[0]) % dn[1]) - j.band_o[1];
                              const int bz = (int)(c / ((long long)dn[0] * dn[1])) - j.band_o[2];
                              if (j.band && (unsigned)bx < (unsigned)j.bs[0] && (unsigned)by < (unsigned)j.bs[1] &&
                                  (unsigned)bz < (unsigned)j.bs[2]) {
                                  const long long nb = (long long)j.bs[0] * j.bs[1] * j.bs[2];
                                  const long long b = bx + (long long)j.bs[0] * (by + (long long)j.bs[1] * bz);
                                  for (int a = 0; a < 3; a++)
                                      v[a] = j.band[(4 + a) * nb + b] + j.fsign * j.band[(7 + a) * nb + b];
                              }
                          }});
    if (j.details) {
        // MORE_DETAILS arrays of OutputVTK (lbm.cpp:2342-2347, 2471-2527)
        arrays.push_back({"Pressure", 1, [&](long long c, const lbm_face *gf, float *v) {
                              v[0] = c >= 0 ? j.det[c] : ghost_pressure(gf);
                          }});
        // a ghost cell's stress is that of its face equilibrium: rho c_s^2 on
        // the diagonal, on xx and yy only for D2Q9 (c_z = 0)
        arrays.push_back({"Viscous Stress", 9, [&](long long c, const lbm_face *gf, float *v) {
                              for (int q = 0; q < 9; q++)
                                  v[q] = c >= 0 ? j.det[(1 + kSym9[q]) * N + c]
                                                : ((q % 4 == 0 && !(j.d2 && q == 8)) ? ghost_stress_diag(gf, j.tau)
                                                                                     : 0.0f);
                          }});
        arrays.push_back({"Vorticity", 3, [&](long long, const lbm_face *, float *) {}});
    }
    if (j.thermal) {
        arrays.push_back({"Temperature", 1, [&](long long c, const lbm_face *gf, float *v) {
                              v[0] = c >= 0 ? j.mom[4 * N + c] : (float)gf->T;
                          }});
        arrays.push_back({"Heat flux", 3, [&](long long c, const lbm_face *, float *v) {
                              if (c >= 0)
                                  for (int a = 0; a < 3; a++) v[a] = j.mom[(5 + a) * N + c];
                          }});
    }
    std::string err;
    if (!write_rectilinear(j.path, j.grid, arrays, err)) {
        o->result = LBM_ERR_INVALID;
        o->error = "output_vtk: " + err;
    }
}
}  // namespace

cudaError_t lbm_mom_acquire(lbm_handle *h) {
    if (h->dl_issued) {
        cudaError_t e = cudaStreamWaitEvent(h->s, h->ev_dl_copied, 0);
        if (e != cudaSuccess) return e;
    }
    if (!h->out || !h->out->copy_issued) return cudaSuccess;
    return cudaStreamWaitEvent(h->s, h->out->copied, 0);
}

void lbm_output_free(lbm_handle *h) {
    lbm_output *o = h->out;
    if (!o) return;
    if (o->writer.joinable()) o->writer.join();
    if (o->copy) cudaStreamSynchronize(o->copy);
    if (o->host) cudaFreeHost(o->host);
    if (o->exported) cudaEventDestroy(o->exported);
    if (o->copied) cudaEventDestroy(o->copied);
    if (o->copy) cudaStreamDestroy(o->copy);
    delete o;
    h->out = nullptr;
}

// D2Q9 handles: the moments (and an IBM body's box force, or in MORE_DETAILS
// mode the pressure and viscous stress) are copied out synchronously, then
// the file is written by the same host thread writer.
static lbm_status output_vtk_2d(lbm_handle *h, const char *path, double u_ref, const uint8_t *types) {
    if (!h->out) h->out = new lbm_output();
    lbm_output *o = h->out;
    lbm_status prev = join_writer(o);
    if (prev != LBM_OK) return prev;
    VtkJob j;
    j.grid = grid_of_2d(h);
    const long long N = j.grid.N;
    const size_t need = (size_t)(h->details ? 8 + LBM_DETAIL_COUNT : 8) * N;
    if (o->host_floats < need) {
        if (o->host) cudaFreeHost(o->host);
        o->host = nullptr;
        o->host_floats = 0;
        if (cudaMallocHost((void **)&o->host, need * sizeof(float)) != cudaSuccess)
            return out_fail(LBM_ERR_NOMEM, "output_vtk: pinned staging allocation failed");
        o->host_floats = need;
    }
    if (h->details) {
        cudaError_t e = l2d_details_async(h, 0, 0.0, 1.0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(o->host + 8 * N, h->det, (size_t)LBM_DETAIL_COUNT * N * sizeof(float),
                                cudaMemcpyDeviceToHost, h->s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
        if (e != cudaSuccess) return out_fail(LBM_ERR_CUDA, std::string("output_vtk: ") + cudaGetErrorString(e));
    }
    lbm_status st = l2d_vtk_snapshot(h, o->host, j.boxF, j.fbox);
    if (st != LBM_OK) return st;
    j.path = path;
    for (int a = 0; a < 3; a++) j.body[a] = (float)h->cfg.body_force[a];
    j.u_ref = u_ref;
    j.tau = h->cfg.tau;
    j.thermal = h->cfg.thermal;
    j.force = l2d_marker_count(h) > 0;
    j.details = h->details ? 1 : 0;
    j.mom = o->host;
    j.band = nullptr;
    j.det = h->details ? o->host + 8 * N : nullptr;
    j.fsign = 1.0f;
    j.d2 = 1;
    j.fcap = (long long)j.boxF.size() / 4;
    j.copied = nullptr;
    if (!grid_types(h, j.grid, types)) return out_fail(LBM_ERR_CUDA, "output_vtk: types");
    o->writer = std::thread(write_vtk, std::move(j), o);
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_output_vtk_async(lbm_handle *h, const char *path, double u_ref, const uint8_t *types) {
    if (!h || !path || !(u_ref > 0.0)) return out_fail(LBM_ERR_INVALID, "output_vtk: bad argument");
    if (!h->inited) return out_fail(LBM_ERR_STATE, "output_vtk: call lbmgpu_init first");
    if (h->d2) return output_vtk_2d(h, path, u_ref, types);
    if (!h->out) {
        h->out = new lbm_output();
        lbm_output *o = h->out;
        if (cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&o->exported, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&o->copied, cudaEventDisableTiming) != cudaSuccess) {
            lbm_output_free(h);
            return out_fail(LBM_ERR_CUDA, "output_vtk: stream/event creation failed");
        }
    }
    lbm_output *o = h->out;
    lbm_status prev = join_writer(o);
    if (prev != LBM_OK) return prev;
    const long long N = h->P.N;
    const int nmom = h->cfg.thermal ? 8 : 5;
    const bool force = h->ibm;
    const size_t nb = force ? (size_t)h->P.nb : 0;
    const size_t ndet = h->details ? (size_t)LBM_DETAIL_COUNT * N : 0;
    const size_t need = (size_t)nmom * N + 12 * nb + ndet;
    if (o->host_floats < need) {
        if (o->host) cudaFreeHost(o->host);
        o->host = nullptr;
        o->host_floats = 0;
        if (cudaMallocHost((void **)&o->host, need * sizeof(float)) != cudaSuccess)
            return out_fail(LBM_ERR_NOMEM, "output_vtk: pinned staging allocation failed");
        o->host_floats = need;
    }
    float *host_band = o->host + (size_t)nmom * N;
    float *host_det = host_band + 12 * nb;
    // snapshot on the main stream: the export pass (and the MORE_DETAILS
    // pass), and the band (small, and rewritten by the next step)
    const cudaError_t ex = h->details ? lbm_details_async(h, 0, 0.0, 1.0) : lbm_export_moments_async(h);
    if (ex != cudaSuccess) return out_fail(LBM_ERR_CUDA, "output_vtk: export failed");
    if (force && cudaMemcpyAsync(host_band, h->band, 12 * nb * sizeof(float), cudaMemcpyDeviceToHost, h->s) !=
                     cudaSuccess)
        return out_fail(LBM_ERR_CUDA, "output_vtk: band copy failed");
    if (cudaEventRecord(o->exported, h->s) != cudaSuccess ||
        cudaStreamWaitEvent(o->copy, o->exported, 0) != cudaSuccess ||
        cudaMemcpyAsync(o->host, h->mom, (size_t)nmom * N * sizeof(float), cudaMemcpyDeviceToHost, o->copy) !=
            cudaSuccess ||
        (ndet && cudaMemcpyAsync(host_det, h->det, ndet * sizeof(float), cudaMemcpyDeviceToHost, o->copy) !=
                     cudaSuccess) ||
        cudaEventRecord(o->copied, o->copy) != cudaSuccess)
        return out_fail(LBM_ERR_CUDA, "output_vtk: copy failed");
    o->copy_issued = true;
    VtkJob j;
    j.path = path;
    j.grid = grid_of(h);
    for (int a = 0; a < 3; a++) j.body[a] = (float)h->cfg.body_force[a];
    j.u_ref = u_ref;
    j.tau = h->cfg.tau;
    j.thermal = h->cfg.thermal;
    j.force = force;
    j.details = h->details;
    j.mom = o->host;
    j.band = force ? host_band : nullptr;
    j.det = h->details ? host_det : nullptr;
    j.fsign = h->icfg.literal_sign ? -1.0f : 1.0f;
    j.bs[0] = h->P.bsx;
    j.bs[1] = h->P.bsy;
    j.bs[2] = h->P.bsz;
    if (force) {
        DevState d;
        if (cudaMemcpyAsync(&d, h->ds, sizeof(d), cudaMemcpyDeviceToHost, h->s) != cudaSuccess ||
            cudaStreamSynchronize(h->s) != cudaSuccess)
            return out_fail(LBM_ERR_CUDA, "output_vtk: state read failed");
        for (int a = 0; a < 3; a++) j.band_o[a] = d.band_o[a];
    }
    if (!grid_types(h, j.grid, types)) return out_fail(LBM_ERR_CUDA, "output_vtk: solid mask read failed");
    j.copied = o->copied;
    o->writer = std::thread(write_vtk, std::move(j), o);
    return LBM_OK;
}

// the moment export's buffer of the handle
static const float *lbm_moment_buffer(lbm_handle *h) { return h->d2 ? l2d_moments(h) : h->mom; }

extern "C" lbm_status lbmgpu_output_avg_vtk(lbm_handle *h, const char *path, double u_ref, const uint8_t *types) {
    if (!h || !path || !(u_ref > 0.0)) return out_fail(LBM_ERR_INVALID, "output_avg_vtk: bad argument");
    if (!h->details) return out_fail(LBM_ERR_STATE, "output_avg_vtk: call lbmgpu_set_more_details first");
    if (!h->inited) return out_fail(LBM_ERR_STATE, "output_avg_vtk: call lbmgpu_init first");
    if (h->out) {
        lbm_status prev = join_writer(h->out);
        if (prev != LBM_OK) return prev;
    }
    const long long N = h->d2 ? l2d_cells(h) : h->P.N;
    std::vector<float> mom((size_t)4 * N), det((size_t)LBM_DETAIL_COUNT * N);
    std::vector<double> st((size_t)LBM_STAT_COUNT * N);
    cudaError_t e = lbm_details_async(h, 0, 0.0, 1.0);
    // the moments as rho, u (3): a D2Q9 export holds rho, ux, uy (uz = 0)
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(mom.data(), lbm_moment_buffer(h), (size_t)(h->d2 ? 3 : 4) * N * sizeof(float),
                            cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(det.data(), h->det, det.size() * sizeof(float), cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st.data(), h->stats, st.size() * sizeof(double), cudaMemcpyDeviceToHost, h->s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->s);
    if (e != cudaSuccess) return out_fail(LBM_ERR_CUDA, std::string("output_avg_vtk: ") + cudaGetErrorString(e));
    VtkGrid g = h->d2 ? grid_of_2d(h) : grid_of(h);
    if (!grid_types(h, g, types)) return out_fail(LBM_ERR_CUDA, "output_avg_vtk: solid mask read failed");
    const double tau = h->cfg.tau, u2 = u_ref * u_ref;
    const bool sampled = h->stat_samples > 0;
    const double told = h->stat_told;
    // a ghost keeps its face state from the first sample on: the averages
    // are that state, the velocity rms and averaged fluctuations zero, the
    // Reynolds-stress rms |u_a u_b| and the pressure rms p sqrt(told / (told + 1))
    auto stat = [&](long long c, int k) { return c >= 0 ? st[(size_t)k * N + c] : 0.0; };
    auto vel = [&](double x) { return (float)((double)(float)x / u_ref); };
    auto rs = [&](double x) { return (float)((double)(float)x / u2); };
    std::vector<VtkArray> arrays;
    arrays.push_back({"Density", 1, [&](long long c, const lbm_face *gf, float *v) {
                          v[0] = c >= 0 ? mom[c] : (float)gf->rho;
                      }});
    arrays.push_back({"Velocity", 3, [&](long long c, const lbm_face *gf, float *v) {
                          for (int a = 0; a < 3; a++) v[a] = c >= 0 ? vel(mom[(1 + a) * N + c]) : vel(gf->u[a]);
                      }});
    arrays.push_back({"Avg velocity", 3, [&](long long c, const lbm_face *gf, float *v) {
                          for (int a = 0; a < 3; a++)
                              v[a] = c >= 0 ? vel(stat(c, LBM_STAT_AVG_U + a)) : (sampled ? vel(gf->u[a]) : 0.0f);
                      }});
    arrays.push_back({"Rms velocity", 3, [&](long long c, const lbm_face *, float *v) {
                          for (int a = 0; a < 3; a++) v[a] = vel(stat(c, LBM_STAT_RMS_U + a));
                      }});
    arrays.push_back({"Pressure", 1, [&](long long c, const lbm_face *gf, float *v) {
                          v[0] = c >= 0 ? det[c] : ghost_pressure(gf);
                      }});
    arrays.push_back({"Avg pressure", 1, [&](long long c, const lbm_face *gf, float *v) {
                          v[0] = c >= 0 ? (float)stat(c, LBM_STAT_AVG_P) : (sampled ? (float)(gf->rho / 3.0) : 0.0f);
                      }});
    arrays.push_back({"Rms pressure", 1, [&](long long c, const lbm_face *gf, float *v) {
                          if (c >= 0) {
                              v[0] = (float)stat(c, LBM_STAT_RMS_P);
                          } else if (sampled) {
                              const double p = gf->rho / 3.0;
                              v[0] = (float)sqrt(p * p * told / (told + 1.0));
                          }
                      }});
    const bool d2 = h->d2 != nullptr;
    arrays.push_back({"Viscous Stress", 9, [&](long long c, const lbm_face *gf, float *v) {
                          for (int q = 0; q < 9; q++)
                              v[q] = c >= 0 ? det[(1 + kSym9[q]) * N + c]
                                            : ((q % 4 == 0 && !(d2 && q == 8)) ? ghost_stress_diag(gf, tau) : 0.0f);
                      }});
    for (const char *name : {"Vorticity", "Avg vorticity", "Rms vorticity"})
        arrays.push_back({name, 3, [&](long long, const lbm_face *, float *) {}});
    arrays.push_back({"Avg reynolds Stress", 9, [&](long long c, const lbm_face *, float *v) {
                          for (int q = 0; q < 9; q++) v[q] = rs(stat(c, LBM_STAT_AVG_RS + kSym9[q]));
                      }});
    arrays.push_back({"Rms reynolds Stress", 9, [&](long long c, const lbm_face *gf, float *v) {
                          static const int ia[9] = {0, 0, 0, 1, 1, 1, 2, 2, 2}, ib[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
                          for (int q = 0; q < 9; q++)
                              v[q] = c >= 0 ? rs(stat(c, LBM_STAT_RMS_RS + kSym9[q]))
                                            : (sampled ? rs(fabs(gf->u[ia[q]] * gf->u[ib[q]])) : 0.0f);
                      }});
    std::string err;
    if (!write_rectilinear(path, g, arrays, err)) return out_fail(LBM_ERR_INVALID, "output_avg_vtk: " + err);
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_output_wait(lbm_handle *h) {
    if (!h) return out_fail(LBM_ERR_INVALID, "output_wait: null handle");
    if (!h->out) return LBM_OK;
    return join_writer(h->out);
}

extern "C" lbm_status lbmgpu_output_markers_vtk(lbm_handle *h, const char *path) {
    if (!h || !path) return out_fail(LBM_ERR_INVALID, "output_markers: bad argument");
    const int n = h->d2 ? l2d_marker_count(h) : (h->ibm ? h->mk.n : 0);
    if (n == 0) return out_fail(LBM_ERR_STATE, "output_markers: no markers set");
    std::vector<double> pos(3 * (size_t)n);
    if (h->d2) {
        const lbm_status st = lbmgpu_get_markers(h, pos.data());
        if (st != LBM_OK) return st;
    } else if (cudaMemcpyAsync(pos.data(), h->mk.pos, pos.size() * sizeof(double), cudaMemcpyDeviceToHost, h->s) !=
                   cudaSuccess ||
               cudaStreamSynchronize(h->s) != cudaSuccess) {
        return out_fail(LBM_ERR_CUDA, "output_markers: copy failed");
    }
    FILE *fp = fopen(path, "w");
    if (!fp) return out_fail(LBM_ERR_INVALID, std::string("output_markers: cannot open ") + path);
    // legacy ASCII POLYDATA; numbers as the reference's stream prints them
    // (6 significant digits); device positions are the reference's node
    // coordinates
    fprintf(fp, "# vtk DataFile Version 3.0\nwall_state\nASCII\nDATASET POLYDATA\n");
    fprintf(fp, "POINTS %d float\n", n);
    for (int m = 0; m < n; m++) fprintf(fp, "%g %g %g \n", pos[m], pos[(size_t)n + m], pos[2 * (size_t)n + m]);
    fprintf(fp, "LINES %d %d\n", n, 3 * n);
    for (int m = 0; m < n; m++) fprintf(fp, "2 %d %d\n", m % n, (m + 1) % n);
    fprintf(fp, "VERTICES 1 %d\n", n + 1);
    fprintf(fp, "%d ", n);
    for (int m = 0; m < n; m++) fprintf(fp, "%d ", m);
    if (fclose(fp) != 0) return out_fail(LBM_ERR_INVALID, std::string("output_markers: write failed: ") + path);
    return LBM_OK;
}

extern "C" lbm_status lbmgpu_output_csv(const char *path, const double *values, int n, double time_step) {
    if (!path || (!values && n > 0) || n < 0) return out_fail(LBM_ERR_INVALID, "output_csv: bad argument");
    FILE *fp = fopen(path, "w");
    if (!fp) return out_fail(LBM_ERR_INVALID, std::string("output_csv: cannot open ") + path);
    fprintf(fp, "time,error\n");
    for (int i = 0; i < n; i++) fprintf(fp, "%g,%g\n", (i + 1) * time_step, values[i]);
    if (fclose(fp) != 0) return out_fail(LBM_ERR_INVALID, std::string("output_csv: write failed: ") + path);
    return LBM_OK;
}
