"""Python mirror of the liblbmgpu C ABI (include/lbmgpu.h), for tests and the bench.

The product is the C-ABI shared library ``liblbmgpu.so`` built from
``csrc/`` (CUDA for sm_103a) and its C++ host facade ``csrc/facade``; this
module only binds the ABI with ctypes.  There is no CPU fallback: if the
library is missing or no GPU is visible, the solver calls fail loudly.

Names follow the reference's LBM class (DestinyFlow01/
Lattice-Boltzmann-Method---Graduate-FSI-, LBM.h:620-664): ``Solver.init``
is LBM::Init, ``Solver.step`` is one Collision + Streaming (+ MacroProp, or
IBLBM first when markers are set), ``Solver.download`` reads the MacroProp
moments.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbmgpu.so")

STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2
STORAGE = {"f32": STORE_F32, "f16": STORE_F16, "bf16": STORE_BF16}
FACE_WALL, FACE_INLET, FACE_OUTLET_EQ, FACE_OUTLET_ZG, FACE_PERIODIC = 0, 1, 2, 3, 4
LATTICE_D3Q19, LATTICE_D2Q9 = 19, 9
# prescribed motion of a D2Q9 IBM body (IBLBM, lbm.cpp:1140-1151)
MOTION_FIXED, MOTION_CONSTANT, MOTION_INLINE_OSC, MOTION_TRANSVERSE_OSC = 0, 1, 2, 3
TWALL_ADIABATIC, TWALL_DIRICHLET, TWALL_NEUMANN = 0, 1, 2
FIELD_RHO, FIELD_UX, FIELD_UY, FIELD_UZ, FIELD_T = 0, 1, 2, 3, 4
FIELD_QX, FIELD_QY, FIELD_QZ = 5, 6, 7
# lbm_config.thermal: none, D3Q7 (D3Q19 handles), the reference's ENERGY model (D2Q9 handles)
THERMAL_NONE, THERMAL_D3Q7, THERMAL_ENERGY = 0, 1, 2
# MORE_DETAILS: the six distinct stress components, and the statistics rows
SYM6 = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))
STAT_AVG_U, STAT_AVG_P, STAT_AVG_RS, STAT_RMS_U, STAT_RMS_P, STAT_RMS_RS, STAT_COUNT = 0, 3, 4, 10, 13, 14, 20
STATUS_RHO_RANGE, STATUS_BAND_EDGE, STATUS_NONFINITE_FORCE, STATUS_TIMEOUT, STATUS_T_RANGE = 1, 2, 4, 16, 32

# Every symbol include/lbmgpu.h declares.
ABI_SYMBOLS = [
    "lbmgpu_config_from_types", "lbmgpu_create", "lbmgpu_destroy", "lbmgpu_init", "lbmgpu_init_fields",
    "lbmgpu_set_markers", "lbmgpu_step", "lbmgpu_step_timed", "lbmgpu_step_profiled", "lbmgpu_download", "lbmgpu_download_f32",
    "lbmgpu_download_all_f32", "lbmgpu_get_forces", "lbmgpu_get_body", "lbmgpu_get_markers", "lbmgpu_status",
    "lbmgpu_sync", "lbmgpu_steps_done", "lbmgpu_device_bytes", "lbmgpu_host_alloc", "lbmgpu_host_free",
    "lbmgpu_last_error", "lbmgpu_abi_version",
    "lbmgpu_batch_create", "lbmgpu_batch_destroy", "lbmgpu_batch_init", "lbmgpu_batch_step",
    "lbmgpu_batch_step_timed", "lbmgpu_batch_autotune", "lbmgpu_batch_download", "lbmgpu_batch_status",
    "lbmgpu_batch_info", "lbmgpu_serve_run", "lbmgpu_batch_step_noalloc", "lbmgpu_step_phases",
    "lbmgpu_set_solids", "lbmgpu_get_solid_forces", "lbmgpu_output_vtk_async", "lbmgpu_output_wait",
    "lbmgpu_output_markers_vtk", "lbmgpu_output_csv", "lbmgpu_save_state", "lbmgpu_load_state",
    "lbmgpu_set_more_details", "lbmgpu_download_details", "lbmgpu_sup_macroprop", "lbmgpu_download_stats",
    "lbmgpu_output_avg_vtk", "lbmgpu_config_from_types_2d", "lbmgpu_set_marker_normals",
    "lbmgpu_config_energy_2d", "lbmgpu_mea_box", "lbmgpu_nusselt", "lbmgpu_download_all_f32_async",
    "lbmgpu_download_wait", "lbmgpu_update_markers", "lbmgpu_cells_per_thread",
    "lbmgpu_energy3d_create", "lbmgpu_energy3d_init", "lbmgpu_energy3d_step", "lbmgpu_energy3d_step_timed",
    "lbmgpu_energy3d_download", "lbmgpu_energy3d_status", "lbmgpu_energy3d_destroy",
]


class Energy3DSetup(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("tau", C.c_double), ("tau_g", C.c_double),
                ("cp", C.c_double), ("g_beta", C.c_double), ("T_star", C.c_double),
                ("type", C.POINTER(C.c_uint8)), ("type_energy", C.POINTER(C.c_uint8)),
                ("T", C.POINTER(C.c_double)), ("rho", C.POINTER(C.c_double)), ("u", C.POINTER(C.c_double)),
                ("F", C.POINTER(C.c_double)), ("graph_steps", C.c_int)]


class Face(C.Structure):
    _fields_ = [("kind", C.c_int), ("thermal_kind", C.c_int), ("rho", C.c_double), ("u", C.c_double * 3),
                ("T", C.c_double)]


class Config(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("tau", C.c_double), ("storage", C.c_int),
                ("faces", Face * 6), ("rho0", C.c_double), ("u0", C.c_double * 3),
                ("body_force", C.c_double * 3), ("thermal", C.c_int), ("tau_g", C.c_double),
                ("T_init", C.c_double), ("T_ref", C.c_double), ("gbeta", C.c_double * 3),
                ("block_x", C.c_int), ("block_y", C.c_int), ("graph_steps", C.c_int), ("staged", C.c_int),
                ("ibm_overlap", C.c_int),
                ("xface", C.c_int), ("lattice", C.c_int), ("cp", C.c_double), ("wall_force", C.c_int),
                ("cells_per_thread", C.c_int)]


class IbmConfig(C.Structure):
    _fields_ = [("n_markers", C.c_int), ("m_max", C.c_int), ("literal_sign", C.c_int), ("free_body", C.c_int),
                ("thermal", C.c_int), ("radius", C.c_double), ("center", C.c_double * 3),
                ("density_ratio", C.c_double), ("volume", C.c_double), ("inertia", C.c_double),
                ("gravity", C.c_double * 3), ("velocity", C.c_double * 3), ("T_body", C.c_double),
                ("free_dofs", C.c_int), ("rho_nearest", C.c_int), ("added_mass", C.c_int), ("motion", C.c_int),
                ("motion_amp", C.c_double), ("motion_freq", C.c_double), ("scheme", C.c_int),
                ("virtual_mass", C.c_double)]


class ServeRequest(C.Structure):
    _fields_ = [("arrival_s", C.c_double), ("kind", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("reynolds", C.c_double), ("steps", C.c_int), ("storage", C.c_int),
                ("fields", C.POINTER(C.c_float))]


class ServeOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("max_active", C.c_int), ("chunk_steps", C.c_int),
                ("time_limit_s", C.c_double), ("sphere_markers", C.c_int), ("m_max", C.c_int)]


class ServeResult(C.Structure):
    _fields_ = [("admit_s", C.c_double), ("finish_s", C.c_double), ("status", C.c_int), ("flags", C.c_uint32),
                ("drag", C.c_double)]


SERVE_CAVITY, SERVE_SPHERE = 0, 1


class LbmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("lbmgpu status %d: %s" % (status, msg))
        self.status = status


_lib = None


def load(path: str | None = None):
    """Load liblbmgpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise OSError("liblbmgpu.so not built at %s (run __graft_entry__.build())" % p)
    L = C.CDLL(p)
    vp, i, d = C.c_void_p, C.c_int, C.c_double
    dp = C.POINTER(C.c_double)
    L.lbmgpu_last_error.restype = C.c_char_p
    L.lbmgpu_abi_version.restype = i
    L.lbmgpu_config_from_types.argtypes = [i, i, i, d, C.POINTER(C.c_uint8), dp, dp, dp, dp, dp, C.POINTER(Config)]
    L.lbmgpu_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
    L.lbmgpu_destroy.argtypes = [vp]
    L.lbmgpu_init.argtypes = [vp]
    L.lbmgpu_init_fields.argtypes = [vp, dp, dp, dp, dp, dp]
    L.lbmgpu_set_markers.argtypes = [vp, C.POINTER(IbmConfig), dp, dp, dp]
    L.lbmgpu_step.argtypes = [vp, i]
    L.lbmgpu_step_timed.argtypes = [vp, i, dp]
    L.lbmgpu_step_profiled.argtypes = [vp, i, dp, dp]
    L.lbmgpu_download.argtypes = [vp, i, dp]
    L.lbmgpu_download_f32.argtypes = [vp, i, C.POINTER(C.c_float)]
    L.lbmgpu_download_all_f32.argtypes = [vp, vp]
    L.lbmgpu_get_forces.argtypes = [vp, dp, i, C.POINTER(i)]
    L.lbmgpu_get_body.argtypes = [vp, dp]
    L.lbmgpu_get_markers.argtypes = [vp, dp]
    L.lbmgpu_status.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.lbmgpu_sync.argtypes = [vp]
    L.lbmgpu_steps_done.argtypes = [vp, C.POINTER(C.c_longlong)]
    L.lbmgpu_device_bytes.argtypes = [vp, C.POINTER(C.c_size_t)]
    L.lbmgpu_cells_per_thread.argtypes = [vp, C.POINTER(C.c_int)]
    L.lbmgpu_host_alloc.argtypes = [C.c_size_t, C.POINTER(vp)]
    L.lbmgpu_host_free.argtypes = [vp]
    L.lbmgpu_batch_create.argtypes = [i, C.POINTER(C.c_int), dp, d, i, C.POINTER(vp)]
    L.lbmgpu_batch_destroy.argtypes = [vp]
    L.lbmgpu_batch_init.argtypes = [vp]
    L.lbmgpu_batch_step.argtypes = [vp, i]
    L.lbmgpu_batch_step_timed.argtypes = [vp, i, dp]
    L.lbmgpu_batch_autotune.argtypes = [vp, C.POINTER(C.c_int)]
    L.lbmgpu_batch_download.argtypes = [vp, i, C.POINTER(C.c_float)]
    L.lbmgpu_batch_status.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.lbmgpu_batch_info.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    L.lbmgpu_step_phases.argtypes = [vp, i, dp]
    L.lbmgpu_set_solids.argtypes = [vp, C.POINTER(C.c_uint8)]
    L.lbmgpu_output_vtk_async.argtypes = [vp, C.c_char_p, d, C.POINTER(C.c_uint8)]
    L.lbmgpu_output_wait.argtypes = [vp]
    L.lbmgpu_save_state.argtypes = [vp, C.c_char_p]
    L.lbmgpu_load_state.argtypes = [vp, C.c_char_p]
    L.lbmgpu_output_markers_vtk.argtypes = [vp, C.c_char_p]
    L.lbmgpu_output_csv.argtypes = [C.c_char_p, dp, i, d]
    L.lbmgpu_set_more_details.argtypes = [vp, i]
    L.lbmgpu_download_details.argtypes = [vp, C.POINTER(C.c_float)]
    L.lbmgpu_sup_macroprop.argtypes = [vp, i, i, d]
    L.lbmgpu_download_stats.argtypes = [vp, dp, C.POINTER(i), dp]
    L.lbmgpu_output_avg_vtk.argtypes = [vp, C.c_char_p, d, C.POINTER(C.c_uint8)]
    L.lbmgpu_config_from_types_2d.argtypes = [i, i, d, C.POINTER(C.c_uint8), dp, dp, dp, C.POINTER(Config)]
    L.lbmgpu_set_marker_normals.argtypes = [vp, dp]
    L.lbmgpu_mea_box.argtypes = [vp, C.POINTER(C.c_int), dp]
    L.lbmgpu_nusselt.argtypes = [vp, d, d, dp]
    L.lbmgpu_energy3d_create.argtypes = [C.POINTER(Energy3DSetup), C.POINTER(vp)]
    L.lbmgpu_energy3d_init.argtypes = [vp]
    L.lbmgpu_energy3d_step.argtypes = [vp, i]
    L.lbmgpu_energy3d_step_timed.argtypes = [vp, i, dp]
    L.lbmgpu_energy3d_download.argtypes = [vp, i, dp]
    L.lbmgpu_energy3d_status.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.lbmgpu_energy3d_destroy.argtypes = [vp]
    L.lbmgpu_download_all_f32_async.argtypes = [vp, vp]
    L.lbmgpu_download_wait.argtypes = [vp]
    L.lbmgpu_update_markers.argtypes = [vp, dp, dp]
    L.lbmgpu_config_energy_2d.argtypes = [C.POINTER(Config), i, i, C.POINTER(C.c_uint8), C.POINTER(C.c_uint8), dp, d,
                                          d]
    L.lbmgpu_get_solid_forces.argtypes = [vp, dp, i, C.POINTER(C.c_int)]
    L.lbmgpu_batch_step_noalloc.argtypes = [i, C.POINTER(C.c_int), dp, d, i, vp, vp, i, i, C.POINTER(C.c_uint32), vp]
    L.lbmgpu_serve_run.argtypes = [C.POINTER(ServeRequest), i, C.POINTER(ServeOptions), C.POINTER(ServeResult), dp]
    for nm in ABI_SYMBOLS:
        fn = getattr(L, nm)
        if fn.restype is None and nm not in ("lbmgpu_last_error", "lbmgpu_abi_version"):
            fn.restype = i
    _lib = L
    return L


def check(status: int):
    if status != 0:
        raise LbmError(status, load().lbmgpu_last_error().decode())


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_config(nx, ny, nz, tau, storage="f32", faces=None, rho0=1.0, u0=(0.0, 0.0, 0.0), body=(0.0, 0.0, 0.0),
                thermal=False, tau_g=0.0, T_init=0.0, T_ref=0.0, gbeta=(0.0, 0.0, 0.0), block=(0, 0),
                graph_steps=0, staged=0, ibm_overlap=0, xface=0, cells=0) -> Config:
    c = Config()
    c.nx, c.ny, c.nz, c.tau = nx, ny, nz, tau
    c.storage = STORAGE[storage] if isinstance(storage, str) else storage
    for f in range(6):
        spec = (faces or {}).get(f, {"kind": FACE_WALL})
        c.faces[f].kind = spec.get("kind", FACE_WALL)
        c.faces[f].thermal_kind = spec.get("thermal_kind", TWALL_ADIABATIC)
        c.faces[f].rho = spec.get("rho", 1.0)
        for a in range(3):
            c.faces[f].u[a] = spec.get("u", (0.0, 0.0, 0.0))[a]
        c.faces[f].T = spec.get("T", 0.0)
    c.rho0 = rho0
    for a in range(3):
        c.u0[a] = u0[a]
        c.body_force[a] = body[a]
        c.gbeta[a] = gbeta[a]
    c.thermal = 1 if thermal else 0
    c.tau_g, c.T_init, c.T_ref = tau_g, T_init, T_ref
    c.block_x, c.block_y = block
    c.graph_steps = graph_steps
    c.staged = staged
    c.ibm_overlap = ibm_overlap
    c.xface = xface
    c.cells_per_thread = cells
    return c


def cavity_config(n, tau=0.8, lid=0.05, storage="f32", ny=None, nz=None, **kw) -> Config:
    """Lid-driven cavity: walls on every face, the y+ face moving with (lid, 0, 0)."""
    faces = {f: {"kind": FACE_WALL} for f in range(6)}
    faces[3] = {"kind": FACE_WALL, "u": (lid, 0.0, 0.0)}
    return make_config(n, ny or n, nz or n, tau, storage, faces, **kw)


def channel_config(nx, ny, nz, tau, u_in=0.05, storage="f32", outlet=FACE_OUTLET_ZG, thermal=False, T_in=0.0,
                   **kw) -> Config:
    """Channel: equilibrium inlet at x-, outlet at x+, bounce-back walls on y and z."""
    faces = {0: {"kind": FACE_INLET, "u": (u_in, 0.0, 0.0), "rho": 1.0, "T": T_in},
             1: {"kind": outlet, "u": (u_in, 0.0, 0.0), "rho": 1.0, "T": T_in}}
    for f in (2, 3, 4, 5):
        faces[f] = {"kind": FACE_WALL}
    return make_config(nx, ny, nz, tau, storage, faces, u0=(u_in, 0.0, 0.0), thermal=thermal, T_init=T_in, **kw)


class Solver:
    """One device-resident solve (an lbm_handle)."""

    def __init__(self, cfg: Config):
        self.L = load()
        self.cfg = cfg
        self.h = C.c_void_p()
        check(self.L.lbmgpu_create(C.byref(cfg), C.byref(self.h)))
        self.shape = (cfg.nz, cfg.ny, cfg.nx)
        self.ncell = cfg.nx * cfg.ny * cfg.nz
        self.n_markers = 0

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.lbmgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self, fields=None):
        if fields is None:
            check(self.L.lbmgpu_init(self.h))
        else:
            arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in fields]
            T = _dp(arrs[4]) if len(arrs) > 4 and arrs[4] is not None else None
            check(self.L.lbmgpu_init_fields(self.h, _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]), _dp(arrs[3]), T))

    def set_markers(self, xyz, ds, radius, center, m_max=5, literal_sign=False, free_body=False, udes=None,
                    density_ratio=0.0, volume=0.0, inertia=0.0, gravity=(0, 0, 0), velocity=(0, 0, 0),
                    thermal=False, T_body=0.0, free_dofs=0, normals=None, rho_nearest=False, added_mass=False,
                    motion=0, motion_amp=0.0, motion_freq=0.0, scheme=0, virtual_mass=0.0):
        """Markers of an immersed body.  The last group of options applies to
        D2Q9 handles (the reference's two-dimensional IBLBM): normals [3][n]
        for the nearest-node density and the added mass, the motion
        (MOTION_*) and the forcing scheme (0 implicit, 1 explicit)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        ds = np.ascontiguousarray(ds, dtype=np.float64)
        n = ds.shape[0]
        ic = IbmConfig()
        ic.n_markers, ic.m_max, ic.literal_sign, ic.free_body = n, m_max, int(literal_sign), int(free_body)
        ic.thermal = int(thermal)
        ic.radius = radius
        for a in range(3):
            ic.center[a] = center[a]
            ic.gravity[a] = gravity[a]
            ic.velocity[a] = velocity[a]
        ic.density_ratio, ic.volume, ic.inertia, ic.T_body = density_ratio, volume, inertia, T_body
        ic.free_dofs = free_dofs
        ic.rho_nearest, ic.added_mass, ic.motion = int(rho_nearest), int(added_mass), int(motion)
        ic.motion_amp, ic.motion_freq, ic.scheme = motion_amp, motion_freq, int(scheme)
        ic.virtual_mass = virtual_mass
        ud = None
        if udes is not None:
            udes = np.ascontiguousarray(udes, dtype=np.float64)
            ud = _dp(udes)
        check(self.L.lbmgpu_set_markers(self.h, C.byref(ic), _dp(xyz), _dp(ds), ud))
        self.n_markers = n
        if normals is not None:
            nrm = np.ascontiguousarray(normals, dtype=np.float64)
            check(self.L.lbmgpu_set_marker_normals(self.h, _dp(nrm)))

    def step(self, n: int = 1):
        check(self.L.lbmgpu_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        ms = C.c_double()
        check(self.L.lbmgpu_step_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def step_profiled(self, n: int):
        tot, fused = C.c_double(), C.c_double()
        check(self.L.lbmgpu_step_profiled(self.h, int(n), C.byref(tot), C.byref(fused)))
        return tot.value, fused.value

    def set_solids(self, mask: np.ndarray):
        """Interior solid cells at rest: mask of shape (nz, ny, nx), non-zero = solid."""
        m = np.ascontiguousarray(np.asarray(mask) != 0, dtype=np.uint8).reshape(-1)
        if m.size != self.ncell:
            raise ValueError("mask must have nx*ny*nz entries")
        check(self.L.lbmgpu_set_solids(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8))))

    def solid_forces(self, max_steps: int = 1 << 16) -> np.ndarray:
        """Rows (Fx, Fy, Fz, step) of the momentum exchange on the solid cells."""
        out = np.zeros((max_steps, 4))
        n = C.c_int()
        check(self.L.lbmgpu_get_solid_forces(self.h, _dp(out), max_steps, C.byref(n)))
        return out[: n.value]

    def mea_box(self, box) -> np.ndarray:
        """MEA_CL / MEA_CD over one box (xmin, xmax, ymin, ymax, zmin, zmax) of
        the reference's ghost-inclusive indices, for the current state (D2Q9
        handles): F = -sum (f*_l + f_opp(l)) c_l; Cd = F[0] / q, Cl = -F[1] / q."""
        b = (C.c_int * 6)(*[int(v) for v in box])
        out = np.zeros(3)
        check(self.L.lbmgpu_mea_box(self.h, b, _dp(out)))
        return out

    def nusselt(self, alpha: float, dT: float) -> float:
        """Find_Nusselt_number of the current state: 1 + <u_y T> / (alpha dT / (Ny + 1))."""
        out = np.zeros(1)
        check(self.L.lbmgpu_nusselt(self.h, alpha, dT, _dp(out)))
        return float(out[0])

    def output_vtk_async(self, path: str, u_ref: float = 1.0, types=None):
        """Write a .vtr of the current state in the reference's layout; returns
        while a host thread writes (see output_wait)."""
        t = None
        if types is not None:
            self._vtk_types = np.ascontiguousarray(types, dtype=np.uint8).ravel()
            t = self._vtk_types.ctypes.data_as(C.POINTER(C.c_uint8))
        check(self.L.lbmgpu_output_vtk_async(self.h, path.encode(), float(u_ref), t))

    # MORE_DETAILS mode (LBM.h:55) ---------------------------------------
    def set_more_details(self, on: bool = True):
        check(self.L.lbmgpu_set_more_details(self.h, 1 if on else 0))

    def details(self) -> dict:
        """Pressure rho/3 and viscous stress (lbm.cpp:681-705) of the current
        state: {"p": [cells], "sigma": [6][cells] in SYM6 order}."""
        out = np.empty((7, self.ncell), dtype=np.float32)
        check(self.L.lbmgpu_download_details(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return {"p": out[0].reshape(self.shape), "sigma": out[1:].reshape((6,) + self.shape)}

    def sup_macroprop(self, n: int, nt: int = 10, dt: float = 1.0):
        """LBM::Sup_MacroProp(n) (lbm.cpp:865-939), told = (n - nt) dt."""
        check(self.L.lbmgpu_sup_macroprop(self.h, int(n), int(nt), float(dt)))

    def stats(self) -> dict:
        out = np.empty((STAT_COUNT, self.ncell), dtype=np.float64)
        n = C.c_int(0)
        told = np.zeros(1)
        check(self.L.lbmgpu_download_stats(self.h, _dp(out), C.byref(n), _dp(told)))
        sh = self.shape
        return {"avg_u": out[0:3].reshape((3,) + sh), "avg_p": out[3].reshape(sh),
                "avg_rs": out[4:10].reshape((6,) + sh), "rms_u": out[10:13].reshape((3,) + sh),
                "rms_p": out[13].reshape(sh), "rms_rs": out[14:20].reshape((6,) + sh), "samples": n.value,
                "told": float(told[0])}

    def output_avg_vtk(self, path: str, u_ref: float = 1.0, types=None):
        t = None
        if types is not None:
            types = np.ascontiguousarray(types, dtype=np.uint8)
            t = types.ctypes.data_as(C.POINTER(C.c_uint8))
        check(self.L.lbmgpu_output_avg_vtk(self.h, path.encode(), float(u_ref), t))

    def save_state(self, path: str):
        check(self.L.lbmgpu_save_state(self.h, path.encode()))

    def load_state(self, path: str):
        check(self.L.lbmgpu_load_state(self.h, path.encode()))

    def output_wait(self):
        check(self.L.lbmgpu_output_wait(self.h))

    def output_markers_vtk(self, path: str):
        check(self.L.lbmgpu_output_markers_vtk(self.h, path.encode()))

    def step_phases(self, n: int) -> dict:
        ph = np.zeros(4)
        check(self.L.lbmgpu_step_phases(self.h, int(n), _dp(ph)))
        return {"total": ph[0], "fused": ph[1], "near": ph[2], "ibm": ph[3]}

    def sync(self):
        check(self.L.lbmgpu_sync(self.h))

    def download(self, field: int) -> np.ndarray:
        out = np.empty(self.ncell, dtype=np.float64)
        check(self.L.lbmgpu_download(self.h, field, _dp(out)))
        return out.reshape(self.shape)

    def download_f32(self, field: int) -> np.ndarray:
        out = np.empty(self.ncell, dtype=np.float32)
        check(self.L.lbmgpu_download_f32(self.h, field, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out.reshape(self.shape)

    def moments(self) -> dict:
        nf = 5 if self.cfg.thermal else 4
        out = np.empty(nf * self.ncell, dtype=np.float32)
        check(self.L.lbmgpu_download_all_f32(self.h, out.ctypes.data_as(C.c_void_p)))
        out = out.reshape((nf,) + self.shape)
        d = {"rho": out[0], "ux": out[1], "uy": out[2], "uz": out[3]}
        if nf == 5:
            d["T"] = out[4]
        return d

    def forces(self, max_steps: int = 1 << 16) -> np.ndarray:
        out = np.zeros((max_steps, 8))
        n = C.c_int()
        check(self.L.lbmgpu_get_forces(self.h, _dp(out), max_steps, C.byref(n)))
        return out[: n.value]

    def body(self) -> np.ndarray:
        out = np.zeros(9)
        check(self.L.lbmgpu_get_body(self.h, _dp(out)))
        return out

    def markers(self) -> np.ndarray:
        out = np.zeros(3 * self.n_markers)
        check(self.L.lbmgpu_get_markers(self.h, _dp(out)))
        return out.reshape(3, self.n_markers)

    def status(self) -> int:
        v = C.c_uint32()
        st = self.L.lbmgpu_status(self.h, C.byref(v))
        if st not in (0, 4):
            check(st)
        return v.value

    def steps_done(self) -> int:
        v = C.c_longlong()
        check(self.L.lbmgpu_steps_done(self.h, C.byref(v)))
        return v.value

    def device_bytes(self) -> int:
        v = C.c_size_t()
        check(self.L.lbmgpu_device_bytes(self.h, C.byref(v)))
        return v.value

    def cells_per_thread(self) -> int:
        """x-cells per thread of the fused step on this solve (1: one cell per thread)."""
        v = C.c_int()
        check(self.L.lbmgpu_cells_per_thread(self.h, C.byref(v)))
        return v.value


def output_csv(path: str, values, time_step: float):
    """OutputCSV: "time,error" rows with time = (i+1) * time_step."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    check(load().lbmgpu_output_csv(path.encode(), _dp(v), int(v.size), float(time_step)))


def read_vtr(path: str) -> dict:
    """Parse a RectilinearGrid .vtr with appended raw data (as OutputVTK
    writes it): header text and every DataArray by name."""
    import re

    raw = open(path, "rb").read()
    cut = raw.index(b'<AppendedData encoding="raw">') + len(b'<AppendedData encoding="raw">')
    head = raw[:cut].decode()
    assert raw[cut:cut + 1] == b"_"
    data = raw[cut + 1:]
    out = {"header": head}
    for m in re.finditer(r'Name="([^"]+)"(?: NumberOfComponents="(\d+)")? format="appended" offset="(\d+)"', head):
        off = int(m.group(3))
        n = int(np.frombuffer(data[off:off + 4], dtype=np.uint32)[0])
        out[m.group(1)] = np.frombuffer(data[off + 4:off + 4 + n], dtype=np.float32).copy()
    return out


def config_from_types(nx, ny, nz, tau, types, rho=None, ux=None, uy=None, uz=None, T=None) -> Config:
    """Reference-style geometry (fluid[..].type incl. ghosts, x fastest) -> Config."""
    L = load()
    t = np.ascontiguousarray(types, dtype=np.uint8).ravel()
    arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (rho, ux, uy, uz, T)]
    ptrs = [None if a is None else _dp(a) for a in arrs]
    cfg = Config()
    check(L.lbmgpu_config_from_types(nx, ny, nz, tau, t.ctypes.data_as(C.POINTER(C.c_uint8)), *ptrs,
                                     C.byref(cfg)))
    return cfg


def config_from_types_2d(nx, ny, tau, types, rho=None, ux=None, uy=None) -> Config:
    """The reference's D2Q9 build (Nz = 1): the computational layer
    fluid[i][j][1] (arrays of (ny+2, nx+2), x fastest) -> a D2Q9 Config."""
    L = load()
    t = np.ascontiguousarray(types, dtype=np.uint8).ravel()
    arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (rho, ux, uy)]
    ptrs = [None if a is None else _dp(a) for a in arrs]
    cfg = Config()
    check(L.lbmgpu_config_from_types_2d(nx, ny, tau, t.ctypes.data_as(C.POINTER(C.c_uint8)), *ptrs, C.byref(cfg)))
    return cfg


def config_energy_2d(cfg: Config, nx, ny, types, types_energy, T, tau_g, cp) -> Config:
    """Add the reference's ENERGY model to a D2Q9 Config made from the same
    (ny+2, nx+2) arrays: type_Energy (TYPE_T = 6 on the walls), the set-up T
    (ghosts included), tau_g and cp (LBM.h:206-214)."""
    L = load()
    t = np.ascontiguousarray(types, dtype=np.uint8).ravel()
    te = np.ascontiguousarray(types_energy, dtype=np.uint8).ravel()
    Ta = np.ascontiguousarray(T, dtype=np.float64).ravel()
    check(L.lbmgpu_config_energy_2d(C.byref(cfg), nx, ny, t.ctypes.data_as(C.POINTER(C.c_uint8)),
                                    te.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(Ta), tau_g, cp))
    return cfg


class Batch:
    """Many lid-driven cavities advanced together (lbmgpu_batch_*)."""

    def __init__(self, dims, taus, lid=0.05, storage="f16"):
        self.L = load()
        self.dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
        self.taus = np.ascontiguousarray(np.asarray(taus, dtype=np.float64))
        self.n = self.dims.shape[0]
        self.h = C.c_void_p()
        st = STORAGE[storage] if isinstance(storage, str) else storage
        check(self.L.lbmgpu_batch_create(self.n, self.dims.ctypes.data_as(C.POINTER(C.c_int)), _dp(self.taus), lid, st,
                                         C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.lbmgpu_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def init(self):
        check(self.L.lbmgpu_batch_init(self.h))

    def step(self, n):
        check(self.L.lbmgpu_batch_step(self.h, int(n)))

    def step_timed(self, n) -> float:
        ms = C.c_double()
        check(self.L.lbmgpu_batch_step_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def autotune(self):
        ch = (C.c_int * 2)()
        check(self.L.lbmgpu_batch_autotune(self.h, ch))
        return ch[0], ch[1]

    def moments(self, p) -> dict:
        nx, ny, nz = (int(v) for v in self.dims[p])
        out = np.empty(4 * nx * ny * nz, dtype=np.float32)
        check(self.L.lbmgpu_batch_download(self.h, p, out.ctypes.data_as(C.POINTER(C.c_float))))
        out = out.reshape(4, nz, ny, nx)
        return {"rho": out[0], "ux": out[1], "uy": out[2], "uz": out[3]}

    def status(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint32)
        check(self.L.lbmgpu_batch_status(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out

    def total_cells(self) -> int:
        v = C.c_longlong()
        check(self.L.lbmgpu_batch_info(self.h, C.byref(v), None))
        return v.value


def serve_run(requests, max_active=32, chunk_steps=50, hbm_budget_bytes=0.0, time_limit_s=0.0, sphere_markers=0,
              m_max=3, keep_fields=False):
    """Run a request trace through lbmgpu_serve_run.  requests: list of dicts
    with arrival_s, kind, nx, ny, nz, reynolds, steps, storage ("f32"/"f16").
    Returns (results list of dicts, lattice updates issued)."""
    L = load()
    n = len(requests)
    arr = (ServeRequest * max(1, n))()
    bufs = []
    for i, r in enumerate(requests):
        a = arr[i]
        a.arrival_s, a.kind = r["arrival_s"], r["kind"]
        a.nx, a.ny, a.nz = r["nx"], r["ny"], r["nz"]
        a.reynolds, a.steps = r["reynolds"], r["steps"]
        st = r.get("storage", "f32")
        a.storage = STORAGE[st] if isinstance(st, str) else st
        if r.get("keep", keep_fields):
            buf = np.zeros(4 * r["nx"] * r["ny"] * r["nz"], dtype=np.float32)
            bufs.append(buf)
            a.fields = buf.ctypes.data_as(C.POINTER(C.c_float))
        else:
            bufs.append(None)
    o = ServeOptions()
    o.hbm_budget_bytes, o.max_active, o.chunk_steps = hbm_budget_bytes, max_active, chunk_steps
    o.time_limit_s, o.sphere_markers, o.m_max = time_limit_s, sphere_markers, m_max
    res = (ServeResult * max(1, n))()
    upd = C.c_double()
    check(L.lbmgpu_serve_run(arr, n, C.byref(o), res, C.byref(upd)))
    out = []
    for i, r in enumerate(requests):
        d = {"admit_s": res[i].admit_s, "finish_s": res[i].finish_s, "status": res[i].status,
             "flags": res[i].flags, "drag": res[i].drag, "latency_s": res[i].finish_s - r["arrival_s"]}
        if bufs[i] is not None:
            d["fields"] = bufs[i].reshape(4, r["nz"], r["ny"], r["nx"])
        out.append(d)
    return out, upd.value


def batch_layout(dims, storage="f16"):
    """Element offsets and strides of the caller-owned population buffers of
    lbmgpu_batch_step_noalloc: S_p = 64 * ceil(N_p / 64), base_p = 19 * sum S_q."""
    dims = np.asarray(dims, dtype=np.int64).reshape(-1, 3)
    N = dims.prod(axis=1)
    S = ((N + 63) // 64) * 64
    base = np.concatenate([[0], np.cumsum(19 * S)[:-1]])
    total = int(19 * S.sum())
    return base, S, total


def batch_step_noalloc(dims, taus, lid, storage, pop_a_ptr, pop_b_ptr, first_step, nsteps, stream=0):
    """Run lbmgpu_batch_step_noalloc on caller-owned device buffers; returns the status words."""
    L = load()
    dims = np.ascontiguousarray(np.asarray(dims, dtype=np.int32).reshape(-1, 3))
    taus = np.ascontiguousarray(np.asarray(taus, dtype=np.float64))
    n = dims.shape[0]
    st = np.zeros(n, dtype=np.uint32)
    check(L.lbmgpu_batch_step_noalloc(n, dims.ctypes.data_as(C.POINTER(C.c_int)), _dp(taus), lid,
                                      STORAGE[storage] if isinstance(storage, str) else storage,
                                      C.c_void_p(pop_a_ptr), C.c_void_p(pop_b_ptr), int(first_step), int(nsteps),
                                      st.ctypes.data_as(C.POINTER(C.c_uint32)), C.c_void_p(stream or None)))
    return st


class Energy3D:
    """The reference's ENERGY model on D3Q19 (its Rayleigh_Benard case), built
    from the reference's ghost-inclusive arrays, shaped (nz+2, ny+2, nx+2)
    like LBM::fluid read k, j, i: type (TYPE_F / TYPE_S), type_Energy (TYPE_T
    Dirichlet, TYPE_Q Neumann, other adiabatic), the set-up T and optionally
    rho, u = (ux, uy, uz) and F = (Fx, Fy, Fz).  g_beta != 0 turns on
    MacroProp's buoyancy F_y = g_beta (T - T_star) on every cell."""

    FIELDS = {"rho": FIELD_RHO, "ux": FIELD_UX, "uy": FIELD_UY, "uz": FIELD_UZ, "T": FIELD_T, "qx": FIELD_QX,
              "qy": FIELD_QY, "qz": FIELD_QZ}

    def __init__(self, types, types_energy, T, tau, tau_g, cp, g_beta=0.0, T_star=0.0, rho=None, u=None, F=None,
                 graph_steps=0):
        self.L = load()
        t = np.ascontiguousarray(types, dtype=np.uint8)
        nz, ny, nx = (d - 2 for d in t.shape)
        self.shape = t.shape
        keep = [t, np.ascontiguousarray(types_energy, dtype=np.uint8), np.ascontiguousarray(T, dtype=np.float64)]
        su = Energy3DSetup(nx=nx, ny=ny, nz=nz, tau=tau, tau_g=tau_g, cp=cp, g_beta=g_beta, T_star=T_star,
                           graph_steps=graph_steps)
        su.type = keep[0].ctypes.data_as(C.POINTER(C.c_uint8))
        su.type_energy = keep[1].ctypes.data_as(C.POINTER(C.c_uint8))
        su.T = _dp(keep[2])
        for name, arr in (("rho", rho), ("u", u), ("F", F)):
            if arr is not None:
                a = np.ascontiguousarray(arr, dtype=np.float64)
                keep.append(a)
                setattr(su, name, _dp(a))
        self.h = C.c_void_p()
        check(self.L.lbmgpu_energy3d_create(C.byref(su), C.byref(self.h)))

    def init(self):
        check(self.L.lbmgpu_energy3d_init(self.h))

    def step(self, n: int):
        check(self.L.lbmgpu_energy3d_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        ms = C.c_double()
        check(self.L.lbmgpu_energy3d_step_timed(self.h, int(n), C.byref(ms)))
        return ms.value

    def download(self, field: str) -> np.ndarray:
        out = np.empty(self.shape)
        check(self.L.lbmgpu_energy3d_download(self.h, self.FIELDS[field], _dp(out)))
        return out

    def moments(self) -> dict:
        return {k: self.download(k) for k in self.FIELDS}

    def status(self) -> int:
        v = C.c_uint32()
        check(self.L.lbmgpu_energy3d_status(self.h, C.byref(v)))
        return int(v.value)

    def close(self):
        if self.h:
            self.L.lbmgpu_energy3d_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
