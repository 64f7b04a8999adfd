// lbm_serve.cu -- continuous-batching request loop over device-resident
// solves (lbmgpu_serve_run).
//
// One host thread.  Requests arrive on a wall-clock schedule; a request is
// admitted (handle created, state initialised on the device) as soon as it
// has arrived, a slot is free and its memory fits the HBM budget, first come
// first served.  Every admitted solve lives on its own CUDA stream and is
// advanced in chunks of steps; a chunk is issued when the solve's previous
// chunk has completed, so many solves' kernels are in flight on the device at
// once and new requests join while others run.  A finished solve is read
// back, its memory released, and its completion time recorded.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lbmgpu.h"
#include "lbm_internal.h"

void lbm_set_last_error(const std::string &m);
cudaStream_t lbm_handle_stream(lbm_handle *h);

namespace {

struct Active {
    int id;
    lbm_handle *h;
    long long issued, total;
    size_t bytes;
    cudaEvent_t ev;
    bool pending;  // a chunk is in flight
};

double now_s(const std::chrono::steady_clock::time_point &t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// Sphere of a channel request: diameter and marker count (the options' count,
// or one marker per unit area, pi D^2).
double sphere_diameter(const lbm_serve_request &r) { return std::max(4.0, std::floor(r.ny / 6.4)); }
int sphere_marker_count(const lbm_serve_request &r, const lbm_serve_options &o) {
    const double D = sphere_diameter(r);
    return o.sphere_markers > 0 ? o.sphere_markers : (int)std::lround(3.14159265 * D * D);
}

// Device bytes of one solve: A/B populations, moments, history and (sphere)
// the band and markers, with 5 % slack.
size_t estimate_bytes(const lbm_serve_request &r, int n_markers) {
    const size_t cells = (size_t)r.nx * r.ny * r.nz;
    const size_t es = r.storage == LBM_STORE_F32 ? 4 : 2;
    size_t b = 2 * 19 * cells * es + 5 * cells * 4 + ((size_t)1 << 16) * 64 + (1 << 20);
    // band of at most 64^3 nodes: 12 FP32 fields and 4 fixed-point accumulators a node
    if (r.kind == LBM_SERVE_SPHERE) b += (size_t)n_markers * 128 + (size_t)(12 * 4 + 4 * 8) * 64 * 64 * 64;
    return b + b / 20;
}

lbm_status start_solve(const lbm_serve_request &r, const lbm_serve_options &o, lbm_handle **out) {
    const double u = 0.05;
    lbm_config c;
    memset(&c, 0, sizeof(c));
    c.nx = r.nx;
    c.ny = r.ny;
    c.nz = r.nz;
    c.storage = r.storage;
    c.rho0 = 1.0;
    for (int f = 0; f < 6; f++) {
        c.faces[f].kind = LBM_FACE_WALL;
        c.faces[f].rho = 1.0;
    }
    double D = 0.0;
    if (r.kind == LBM_SERVE_CAVITY) {
        // lid-driven cavity, Re on the lid velocity and the x edge
        c.tau = 0.5 + 3.0 * u * r.nx / r.reynolds;
        c.faces[3].u[0] = u;
    } else {
        // channel with a fixed sphere, Re on the inflow velocity and D
        D = sphere_diameter(r);
        c.tau = 0.5 + 3.0 * u * D / r.reynolds;
        c.faces[0].kind = LBM_FACE_INLET;
        c.faces[0].u[0] = u;
        c.faces[1].kind = LBM_FACE_OUTLET_ZG;
        c.faces[1].u[0] = u;
        c.u0[0] = u;
    }
    lbm_status s = lbmgpu_create(&c, out);
    if (s != LBM_OK) return s;
    if ((s = lbmgpu_init(*out)) != LBM_OK) return s;
    if (r.kind == LBM_SERVE_SPHERE) {
        const int n = sphere_marker_count(r, o);
        const double R = D / 2.0, cen[3] = {r.nx / 4.0, r.ny / 2.0, r.nz / 2.0};
        const double ga = 3.14159265 * (3.0 - std::sqrt(5.0));
        std::vector<double> xyz(3 * (size_t)n), ds(n, 3.14159265 * D * D / n);
        for (int m = 0; m < n; m++) {
            const double zz = 1.0 - (2.0 * m + 1.0) / n, rr = std::sqrt(1.0 - zz * zz), ph = ga * m;
            xyz[m] = cen[0] + R * rr * std::cos(ph);
            xyz[n + m] = cen[1] + R * rr * std::sin(ph);
            xyz[2 * (size_t)n + m] = cen[2] + R * zz;
        }
        lbm_ibm_config ic;
        memset(&ic, 0, sizeof(ic));
        ic.n_markers = n;
        ic.m_max = o.m_max > 0 ? o.m_max : 3;
        ic.radius = R;
        for (int a = 0; a < 3; a++) ic.center[a] = cen[a];
        if ((s = lbmgpu_set_markers(*out, &ic, xyz.data(), ds.data(), nullptr)) != LBM_OK) return s;
    }
    return LBM_OK;
}

}  // namespace

extern "C" lbm_status lbmgpu_serve_run(const lbm_serve_request *reqs, int n, const lbm_serve_options *opt,
                                       lbm_serve_result *out, double *lattice_updates) {
    if (!reqs || !opt || !out || n < 0) {
        lbm_set_last_error("serve_run: null argument");
        return LBM_ERR_INVALID;
    }
    const lbm_serve_options o = *opt;
    const int max_active = std::max(1, o.max_active);
    const int chunk = std::max(1, o.chunk_steps);
    for (int i = 0; i < n; i++) {
        out[i].admit_s = -1.0;
        out[i].finish_s = -1.0;
        out[i].status = LBM_OK;
        out[i].flags = 0;
        out[i].drag = 0.0;
        if (i > 0 && reqs[i].arrival_s < reqs[i - 1].arrival_s) {
            lbm_set_last_error("serve_run: requests must be sorted by arrival time");
            return LBM_ERR_INVALID;
        }
    }
    std::vector<Active> act;
    size_t used = 0;
    int next = 0, done = 0;
    double updates = 0.0;
    const auto t0 = std::chrono::steady_clock::now();
    while (done < n) {
        const double t = now_s(t0);
        bool progressed = false;
        const bool closed = o.time_limit_s > 0 && t > o.time_limit_s;
        // admission, first come first served
        while (!closed && next < n && reqs[next].arrival_s <= t && (int)act.size() < max_active) {
            const lbm_serve_request &r = reqs[next];
            const size_t need = estimate_bytes(r, sphere_marker_count(r, o));
            if (o.hbm_budget_bytes > 0 && used + need > (size_t)o.hbm_budget_bytes) {
                if (act.empty()) {  // can never fit: reject instead of waiting forever
                    out[next].status = LBM_ERR_NOMEM;
                    done++;
                    next++;
                    continue;
                }
                break;
            }
            Active a;
            a.id = next;
            a.h = nullptr;
            a.issued = 0;
            a.total = std::max(0, r.steps);
            a.bytes = need;
            a.pending = false;
            lbm_status s = start_solve(r, o, &a.h);
            if (s == LBM_OK && cudaEventCreateWithFlags(&a.ev, cudaEventDisableTiming) != cudaSuccess)
                s = LBM_ERR_CUDA;
            out[next].admit_s = now_s(t0);
            if (s != LBM_OK) {
                out[next].status = s;
                out[next].finish_s = now_s(t0);
                if (a.h) lbmgpu_destroy(a.h);
                done++;
            } else {
                used += need;
                act.push_back(a);
            }
            next++;
            progressed = true;
        }
        if (closed) {
            // no more admissions: count the requests that never got a slot
            while (next < n) {
                out[next].status = LBM_ERR_STATE;
                next++;
                done++;
            }
        }
        // issue chunks, retire finished solves
        for (size_t i = 0; i < act.size();) {
            Active &a = act[i];
            if (a.pending) {
                cudaError_t q = cudaEventQuery(a.ev);
                if (q == cudaErrorNotReady) {
                    i++;
                    continue;
                }
                a.pending = false;
                if (q != cudaSuccess) out[a.id].status = LBM_ERR_CUDA;
            }
            if (out[a.id].status == LBM_OK && a.issued < a.total && !closed) {
                const int c = (int)std::min<long long>(chunk, a.total - a.issued);
                lbm_status s = lbmgpu_step(a.h, c);
                if (s == LBM_OK && cudaEventRecord(a.ev, lbm_handle_stream(a.h)) == cudaSuccess) {
                    a.issued += c;
                    a.pending = true;
                    updates += (double)reqs[a.id].nx * reqs[a.id].ny * reqs[a.id].nz * c;
                    progressed = true;
                    i++;
                    continue;
                }
                out[a.id].status = s == LBM_OK ? LBM_ERR_CUDA : s;
            }
            // finished (or failed): read back and release
            const lbm_serve_request &r = reqs[a.id];
            uint32_t flags = 0;
            lbm_status st = lbmgpu_status(a.h, &flags);
            out[a.id].flags = flags;
            if (out[a.id].status == LBM_OK && st != LBM_OK) out[a.id].status = st;
            if (a.issued < a.total && out[a.id].status == LBM_OK) out[a.id].status = LBM_ERR_STATE;
            if (r.fields && out[a.id].status == LBM_OK) out[a.id].status = lbmgpu_download_all_f32(a.h, r.fields);
            if (r.kind == LBM_SERVE_SPHERE) {
                double f[8];
                int got = 0;
                if (lbmgpu_get_forces(a.h, f, 1, &got) == LBM_OK && got == 1) out[a.id].drag = f[0];
            }
            out[a.id].finish_s = now_s(t0);
            cudaEventDestroy(a.ev);
            lbmgpu_destroy(a.h);
            used -= a.bytes;
            done++;
            act[i] = act.back();
            act.pop_back();
            progressed = true;
        }
        if (!progressed) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    if (lattice_updates) *lattice_updates = updates;
    return LBM_OK;
}
