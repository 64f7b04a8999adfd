"""FP64 CPU oracle for the LBM hot path (test infrastructure only).

This package is the test oracle the GPU results are compared with.  The CUDA product path never imports
it; only ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` use it.

* ``lbm_oracle.c``   -- plain-C FP64 restatement of the reference time step
  (Init, Collision/ConvLBM, Streaming, MacroProp, IBLBM, ...), each function
  citing the reference ``lbm.cpp`` lines it follows.
* ``build_ref.sh``   -- recipe that compiles the reference's own ``lbm.cpp``
  (unmodified, where it lies) with ``ref_config.h`` + ``ref_harness.cpp`` into
  ``oracle/_ref/``; used to pin the restatement (``tests/golden``).

This module loads the restatement with ctypes and builds the benchmark cases
(3D cavity, channel with an immersed sphere, 2D IBM cylinder) as numpy-backed
lattices.  Arrays are indexed ``[k, j, i]`` (x fastest), ghost layers
included.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liblbm_oracle.so")

TYPE_F, TYPE_S, TYPE_OUT, TYPE_IN, TYPE_P, TYPE_L, TYPE_T, TYPE_Q, TYPE_OUTZG = 0, 1, 2, 3, 4, 5, 6, 7, 8

# D3Q19 in the reference order (LBM.h:542-552)
CX19 = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0])
CY19 = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 1, -1])
CZ19 = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, -1, 1, -1, 1])
W19 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
# D2Q9 in the reference order (LBM.h:533-537)
CX9 = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY9 = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
CZ9 = np.zeros(9, dtype=np.int64)
REF_PI = 3.14159265


def build(force: bool = False) -> str:
    """Compile lbm_oracle.c into oracle/_build/liblbm_oracle.so (gcc, OpenMP)."""
    src = os.path.join(HERE, "lbm_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", tmp, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


# Where this build environment keeps the reference tree (read-only); the
# environment variable REF overrides it.  Absent on hosts that only run the
# prebuilt files.
REF_TREE = os.environ.get("REF", "/root/reference")


def build_ref(*variants: str) -> None:
    """Run the reference-literal recipe (no-op when the reference tree is absent)."""
    env = dict(os.environ, REF=REF_TREE)
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"), *variants], env=env)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, d, i, l = C.c_void_p, C.c_double, C.c_int, C.c_long
        L.orc_create.restype = vp
        L.orc_create.argtypes = [i, i, i, i, d]
        L.orc_free.argtypes = [vp]
        L.orc_enable_thermal.argtypes = [vp, d, d, d, d, d]
        L.orc_enable_energy.argtypes = [vp, d, d, d]
        L.orc_energy_buoyancy.argtypes = [vp, d, d]
        L.orc_force_all.argtypes = [vp, i]
        L.orc_types_energy.restype = C.POINTER(C.c_uint8)
        L.orc_types_energy.argtypes = [vp]
        L.orc_ncell.restype = l
        L.orc_ncell.argtypes = [vp]
        L.orc_types.restype = C.POINTER(C.c_uint8)
        L.orc_types.argtypes = [vp]
        L.orc_field.restype = C.POINTER(C.c_double)
        L.orc_field.argtypes = [vp, i]
        L.orc_set_body_force.argtypes = [vp, d, d, d]
        L.orc_feq.restype = d
        L.orc_feq.argtypes = [vp, d, d, d, d, i]
        L.orc_init.argtypes = [vp]
        L.orc_mea.argtypes = [vp, i, i, i, i, i, i, C.POINTER(C.c_double)]
        L.orc_collide.restype = l
        L.orc_collide.argtypes = [vp]
        L.orc_stream.argtypes = [vp]
        L.orc_macro.restype = l
        L.orc_macro.argtypes = [vp]
        L.orc_step_plain.restype = l
        L.orc_step_plain.argtypes = [vp, i]
        L.orc_kernel.restype = d
        L.orc_kernel.argtypes = [d]
        L.orc_ibm_step.argtypes = [vp, vp, vp, C.POINTER(d), C.POINTER(d)]
        L.orc_step_ibm.restype = l
        L.orc_step_ibm.argtypes = [vp, vp, vp, C.POINTER(d), C.POINTER(d)]
        L.orc_fibonacci_sphere.argtypes = [i, d, C.POINTER(d)] + [C.POINTER(d)] * 7
        L.orc_body_step.argtypes = [vp, vp, d, C.POINTER(d), C.POINTER(d)]
        L.orc_internal_momentum.argtypes = [vp, C.POINTER(d), d, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(d)]
        L.orc_nusselt_volume.restype = d
        L.orc_nusselt_volume.argtypes = [vp, d, d]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Markers(C.Structure):
    """Mirror of ``orc_markers``; numpy arrays own the memory."""

    _fields_ = [("n", C.c_int)] + [
        (nm, C.POINTER(C.c_double))
        for nm in ("x", "y", "z", "nx", "ny", "nz", "ds", "udx", "udy", "udz", "ubx", "uby", "ubz",
                   "Fbx", "Fby", "Fbz", "Td", "Tb", "Qb")
    ]

    def __init__(self, n: int):
        super().__init__()
        self.n = n
        self.arrays = {}
        for nm, _ in self._fields_[1:]:
            a = np.zeros(n)
            self.arrays[nm] = a
            setattr(self, nm, _dp(a))

    def __getitem__(self, nm):
        return self.arrays[nm]


class IbmOpts(C.Structure):
    """Mirror of ``orc_ibm_opts``."""

    _fields_ = [("box_lo", C.c_int * 3), ("box_hi", C.c_int * 3), ("m_max", C.c_int),
                ("lit_sign", C.c_int), ("rho_mode", C.c_int), ("thermal", C.c_int),
                ("use_avg_density", C.c_int), ("vsolid", C.c_double),
                ("vcm_new", C.c_double * 3), ("vcm_old", C.c_double * 3), ("scheme", C.c_int)]


class Body(C.Structure):
    """Mirror of ``orc_body``."""

    _fields_ = [("xc", C.c_double * 3), ("v", C.c_double * 3), ("om", C.c_double * 3),
                ("rho_ratio", C.c_double), ("vol", C.c_double), ("inertia", C.c_double),
                ("grav", C.c_double * 3), ("dof", C.c_int), ("have_prev", C.c_int),
                ("internal_prev", C.c_double * 6), ("cv", C.c_double), ("v_prev", C.c_double * 3),
                ("om_prev", C.c_double * 3)]


class Lattice:
    """An FP64 lattice of (nx+2)(ny+2)(nz+2) cells, ghost layers included."""

    def __init__(self, q: int, nx: int, ny: int, nz: int, tau: float):
        self.L = lib()
        self.q, self.nx, self.ny, self.nz, self.tau = q, nx, ny, nz, tau
        self.h = self.L.orc_create(q, nx, ny, nz, tau)
        self.shape = (nz + 2, ny + 2, nx + 2)
        self.n = int(self.L.orc_ncell(self.h))
        self.thermal = False
        self.energy = False

    def __del__(self):
        try:
            if self.h:
                self.L.orc_free(self.h)
                self.h = None
        except Exception:
            pass

    def enable_thermal(self, tau_g: float, T0: float = 0.0, gbeta=(0.0, 0.0, 0.0)):
        self.L.orc_enable_thermal(self.h, tau_g, T0, *gbeta)
        self.thermal = True

    def enable_energy(self, tau_g: float, cp: float, nu: float):
        """The reference's ENERGY model: g on the flow lattice (q
        populations), viscous heating with cp and nu, Dirichlet walls where
        ``types_energy`` is TYPE_T.  Set T (walls included) before init()."""
        self.L.orc_enable_energy(self.h, tau_g, cp, nu)
        self.energy = True

    def force_on_every_cell(self, on: bool = True):
        """Poiseuille_Flow's MacroProp: the body force set on every cell, walls
        included (lbm.cpp:800-801), so walls report u = F / 2 from the second
        MacroProp on and count as moving."""
        self.L.orc_force_all(self.h, int(on))

    def energy_buoyancy(self, g_beta: float, T_star: float):
        """Rayleigh_Benard: F_y = g_beta (T - T_star) on every cell."""
        self.L.orc_energy_buoyancy(self.h, g_beta, T_star)

    @property
    def types_energy(self) -> np.ndarray:
        p = self.L.orc_types_energy(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n,)).reshape(self.shape)

    def _view(self, which: int, comps: int = 1) -> np.ndarray:
        p = self.L.orc_field(self.h, which)
        a = np.ctypeslib.as_array(p, shape=(comps * self.n,))
        if comps == 1:
            return a.reshape(self.shape)
        return a.reshape((comps,) + self.shape)

    @property
    def types(self) -> np.ndarray:
        p = self.L.orc_types(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n,)).reshape(self.shape)

    rho = property(lambda s: s._view(0))
    ux = property(lambda s: s._view(1))
    uy = property(lambda s: s._view(2))
    uz = property(lambda s: s._view(3))
    Fx = property(lambda s: s._view(4))
    Fy = property(lambda s: s._view(5))
    Fz = property(lambda s: s._view(6))
    f = property(lambda s: s._view(7, s.q))
    fs = property(lambda s: s._view(8, s.q))
    T = property(lambda s: s._view(9))
    g = property(lambda s: s._view(10, 7))
    gs = property(lambda s: s._view(11, 7))
    eg = property(lambda s: s._view(13, s.q))
    hq = property(lambda s: s._view(14, 3))
    egs = property(lambda s: s._view(15, s.q))
    fvis = property(lambda s: s._view(16, s.q))

    def set_body_force(self, fx, fy, fz):
        self.L.orc_set_body_force(self.h, fx, fy, fz)

    def init(self):
        self.L.orc_init(self.h)

    def step_plain(self, n: int) -> int:
        return int(self.L.orc_step_plain(self.h, n))

    def collide(self) -> int:
        return int(self.L.orc_collide(self.h))

    def stream(self):
        self.L.orc_stream(self.h)

    def macro(self) -> int:
        return int(self.L.orc_macro(self.h))

    def interior(self, a: np.ndarray) -> np.ndarray:
        return a[1:-1, 1:-1, 1:-1] if self.nz > 1 or a.shape[0] > 1 else a

    def mea(self, box) -> np.ndarray:
        """Momentum-exchange sums (x, y, z) over the fluid cells of box =
        (xmin, xmax, ymin, ymax, zmin, zmax), ghost-inclusive indices."""
        out = np.zeros(3)
        self.L.orc_mea(self.h, *[int(b) for b in box], _dp(out))
        return out

    def ibm_step(self, mk: Markers, op: IbmOpts, center) -> np.ndarray:
        c = np.ascontiguousarray(center, dtype=np.float64)
        out = np.zeros(7)
        self.L.orc_ibm_step(self.h, C.byref(mk), C.byref(op), _dp(c), _dp(out))
        return out

    def step_ibm(self, mk: Markers, op: IbmOpts, center) -> np.ndarray:
        c = np.ascontiguousarray(center, dtype=np.float64)
        out = np.zeros(7)
        self.L.orc_step_ibm(self.h, C.byref(mk), C.byref(op), _dp(c), _dp(out))
        return out


# --------------------------------------------------------------------------
# Case builders
# --------------------------------------------------------------------------

def cavity(n: int, tau: float = 0.8, lid: float = 0.05, ny: int | None = None, nz: int | None = None) -> Lattice:
    """D3Q19 lid-driven cavity: ghost walls TYPE_S, the ghost plane j = Ny+1
    moving with u = (lid, 0, 0) (Couette top-wall convention,
    lbm.cpp:1548-1551); rho = 1, u = 0 inside, f = feq."""
    nx = n
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    lat = Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_S
    t[1:-1, 1:-1, 1:-1] = TYPE_F
    lat.ux[:, -1, :] = lid
    lat.init()
    return lat


def channel(nx: int, ny: int, nz: int, tau: float, u_in: float = 0.05, outlet: int = TYPE_OUTZG) -> Lattice:
    """D3Q19 channel: inlet ghost plane x = 0 (TYPE_IN, equilibrium at u_in),
    outlet ghost plane x = nx+1 (zero-gradient by default), halfway
    bounce-back walls on the y and z ghost planes (walls take the edges).
    Initial state: rho = 1, u = (u_in, 0, 0) everywhere (lbm.cpp:1804-1818)."""
    lat = Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    t[:, :, 0] = TYPE_IN
    t[:, :, -1] = outlet
    t[:, 0, :] = TYPE_S
    t[:, -1, :] = TYPE_S
    t[0, :, :] = TYPE_S
    t[-1, :, :] = TYPE_S
    fluidlike = t != TYPE_S
    lat.ux[fluidlike] = u_in
    lat.init()
    return lat


def sphere_bb(nx: int, ny: int, nz: int, tau: float, diameter: float, u_max: float = 0.1):
    """The reference's staircase sphere (main_setup_Sphere / Generate_Sphere,
    lbm.cpp:1759-1822): cells whose centre (i - 1/2, j - 1/2, k - 1/2) lies
    within D/2 of (Nx/5, Ny/2, Nz/2) are TYPE_S at rest; ghost plane x = 0
    TYPE_IN, every other ghost plane TYPE_OUT; fluid-like cells start at
    rho = 1, u = (u_max, 0, 0).  Returns (lattice, MEA box)."""
    lat = Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    c = (nx / 5.0, ny / 2.0, nz / 2.0)
    k, j, i = np.meshgrid(np.arange(nz + 2), np.arange(ny + 2), np.arange(nx + 2), indexing="ij")
    r = np.sqrt((c[0] - (i - 0.5)) ** 2 + (c[1] - (j - 0.5)) ** 2 + (c[2] - (k - 0.5)) ** 2)
    inside = (r <= diameter / 2.0) & (i >= 1) & (i <= nx) & (j >= 1) & (j <= ny) & (k <= nz)
    t[inside] = TYPE_S
    t[:, :, 0] = TYPE_IN
    t[:, :, -1] = TYPE_OUT
    t[:, 0, :] = TYPE_OUT
    t[:, -1, :] = TYPE_OUT
    t[0, :, :] = TYPE_OUT
    t[-1, :, :] = TYPE_OUT
    lat.rho[:] = 1.0
    lat.ux[t != TYPE_S] = u_max
    lat.init()
    box = (int(c[0] - diameter), int(c[0] + diameter), int(c[1] - diameter), int(c[1] + diameter),
           int(c[2] - diameter), int(c[2] + diameter))
    return lat, box


def _ctrunc(v: float) -> int:
    """C's double -> int conversion (truncation toward zero)."""
    return int(v)


def staircase2d(kind: str, nx: int, ny: int, D: float, Re: float, u_max: float, lpd: float = 1.5, nb: int = 1):
    """The reference's staircase 2D bodies with momentum-exchange Cl/Cd, set
    up as its own code does (D2Q9, Nz = 1, ghost-inclusive grid):
      "cylbasic"  Cylinder_Basic (Generate_Cylinder / main_setup_Cylinder,
                  lbm.cpp:1429-1494): cells whose centre (i - 1/2, j - 1/2)
                  lies within D/2 of (Nx/5, Ny/2), i, j in 1..N;
      "tandem"    Cylinder_Tandem_Circle (lbm.cpp:1645-1704): nb circles of
                  the integer diameter D (radius D/2 in integer division) at
                  (Nx/5, Ny/2 + L/2 - n L), L = lpd D, the centres taken as
                  int;
      "triangle"  Cylinder_Tandem_Triangle (lbm.cpp:1706-1757): nb
                  equilateral triangles, tip (Nx/5 + n L, Ny/2), columns
                  i = 0..D with rows floor(-i/sqrt 3)..ceil(i/sqrt 3).
    Ghost faces and initial state follow each set-up, including the order
    in which the faces are assigned (it decides the corner ghosts).
    tau = 0.5 + u_max D / Re / cs2.  Returns (lattice, MEA boxes in the
    reference's indices, reference area A of C = F / (0.5 rho0 U^2 A))."""
    cs2 = 1.0 / 3.0
    tau = 0.5 + (u_max * D / Re) / cs2
    lat = Lattice(9, nx, ny, 1, tau)
    t = lat.types  # [k][j][i]
    t[:] = TYPE_F
    NX, NY = nx + 2, ny + 2
    boxes = []
    if kind == "cylbasic":
        cx, cy = nx / 5.0, ny / 2.0
        for k in (0, 1):
            for j in range(1, ny + 1):
                for i in range(1, nx + 1):
                    if np.sqrt((cx - (i - 0.5)) ** 2 + (cy - (j - 0.5)) ** 2) <= D / 2.0:
                        t[k, j, i] = TYPE_S
        t[:, :, 0] = TYPE_IN
        t[:, :, -1] = TYPE_OUT
        t[:, 0, :] = TYPE_OUT
        t[:, -1, :] = TYPE_OUT
        fluid = t != TYPE_S
        boxes.append((_ctrunc(cx - D), _ctrunc(cx + D), _ctrunc(cy - D), _ctrunc(cy + D)))
        area = D
    elif kind == "tandem":
        Di = int(D)
        L = Di * lpd
        cx = nx // 5
        cy0 = _ctrunc(ny // 2 + L / 2)
        rad = float(Di // 2)
        for n in range(nb):
            cy = _ctrunc(cy0 - n * L)
            for i in range(cx - Di, cx + Di + 1):
                for j in range(cy - Di, cy + Di + 1):
                    if np.sqrt((cx - (i - 0.5)) ** 2 + (cy - (j - 0.5)) ** 2) <= rad:
                        t[0:2, j, i] = TYPE_S
            boxes.append((_ctrunc(cx - L / 2), _ctrunc(cx + L / 2), _ctrunc(cy0 - n * L - L / 2),
                          _ctrunc(cy0 - n * L + L / 2)))
        t[:, 0, :] = TYPE_OUT
        t[:, -1, :] = TYPE_OUT
        t[:, :, 0] = TYPE_IN
        t[:, :, -1] = TYPE_OUT
        fluid = t != TYPE_S
        area = float(Di)
    elif kind == "triangle":
        Di = int(D)
        L = Di * lpd
        tx, ty = nx // 5, ny // 2
        for n in range(nb):
            tip = _ctrunc(tx + n * L)
            for i in range(Di + 1):
                for j in range(int(np.floor(-i / np.sqrt(3))), int(np.ceil(i / np.sqrt(3))) + 1):
                    t[:, ty + j, tip + i] = TYPE_S
            boxes.append((_ctrunc(tx + n * L - Di // 4), _ctrunc(tx + n * L + (Di + L) / 2), ty - Di, ty + Di))
        t[:, 0, :] = TYPE_OUT
        t[:, -1, :] = TYPE_OUT
        t[:, :, 0] = TYPE_IN
        t[:, :, -1] = TYPE_OUT
        t[0, :, :] = TYPE_F
        t[-1, :, :] = TYPE_F
        fluid = t != TYPE_S
        area = 2.0 * Di / np.sqrt(3.0)
    else:
        raise ValueError(kind)
    lat.rho[:] = 1.0
    lat.ux[fluid] = u_max
    lat.init()
    return lat, boxes, area


def staircase2d_run(kind: str, nx: int, ny: int, D: float, Re: float, u_max: float, steps: int, lpd: float = 1.5,
                    nb: int = 1):
    """Run a staircase case for `steps` steps in the reference order
    (Collision, Streaming, MacroProp; main.cpp:214-220), taking MEA_CL /
    MEA_CD (lbm.cpp:3085-3163) in every box after every step.  Returns
    (lattice, cl[nb][steps], cd[nb][steps])."""
    lat, boxes, area = staircase2d(kind, nx, ny, D, Re, u_max, lpd, nb)
    q = 0.5 * 1.0 * u_max * u_max * area
    cl = np.zeros((len(boxes), steps))
    cd = np.zeros((len(boxes), steps))
    for s_ in range(steps):
        assert lat.step_plain(1) == 0
        for b, (x0, x1, y0, y1) in enumerate(boxes):
            m = lat.mea((x0, x1, y0, y1, 1, 1))
            cl[b, s_] = m[1] / q
            cd[b, s_] = -m[0] / q
    return lat, cl, cd


def fibonacci_sphere(n: int, diameter: float, center) -> Markers:
    mk = Markers(n)
    c = np.ascontiguousarray(center, dtype=np.float64)
    a = mk.arrays
    lib().orc_fibonacci_sphere(n, diameter / 2.0, _dp(c), _dp(a["x"]), _dp(a["y"]), _dp(a["z"]),
                               _dp(a["nx"]), _dp(a["ny"]), _dp(a["nz"]), _dp(a["ds"]))
    return mk


def sphere_box(center, diameter: float, lat: Lattice) -> tuple:
    """Eulerian node box covering every marker stencil: [floor(c - R) - 2,
    ceil(c + R) + 2], clamped to the lattice (ghosts included)."""
    R = diameter / 2.0
    lo, hi = [], []
    lims = (lat.nx + 1, lat.ny + 1, lat.nz + 1)
    for a in range(3):
        lo.append(max(0, int(np.floor(center[a] - R)) - 2))
        hi.append(min(lims[a], int(np.ceil(center[a] + R)) + 2))
    return lo, hi


def ibm_opts(lo, hi, m_max: int, lit_sign: int = 0, rho_mode: int = 0, thermal: int = 0) -> IbmOpts:
    op = IbmOpts()
    for a in range(3):
        op.box_lo[a] = lo[a]
        op.box_hi[a] = hi[a]
    op.m_max = m_max
    op.lit_sign = lit_sign
    op.rho_mode = rho_mode
    op.thermal = thermal
    op.use_avg_density = 0
    return op


def cylinder_markers_literal(nodes: int, D: float, cx: float, cy: float) -> Markers:
    """Generate_Cylinder_Marker (lbm.cpp:1857-1877) + Normal_Marker
    (lbm.cpp:1048-1069) + ds (main.cpp:123-131), restated."""
    mk = Markers(nodes)
    a = mk.arrays
    r = D / 2.0
    i = np.arange(nodes)
    a["x"][:] = r * np.cos(2 * REF_PI / nodes * i) + cx + 0.5
    a["y"][:] = r * np.sin(2 * REF_PI / nodes * i) + cy + 0.5
    a["z"][:] = 1.0
    x2 = np.roll(a["x"], -1)
    y2 = np.roll(a["y"], -1)
    ddx, ddy = x2 - a["x"], y2 - a["y"]
    norm = np.sqrt(ddx ** 2 + ddy ** 2 + 0.0 ** 2)
    tx, ty = ddx / norm, ddy / norm
    a["nx"][:] = ty * 1 - 0.0 * 0
    a["ny"][:] = 0.0 * 0 - tx * 1
    a["nz"][:] = tx * 0 - ty * 0
    a["ds"][:] = np.sqrt((a["x"] - x2) ** 2 + (a["y"] - y2) ** 2 + 0.0)
    return mk


def couette_energy(ny: int, Re: float, tau: float = 0.9, nx: int = 2, nz: int = 2, Pr: float = 0.7,
                   Br: float = 10.0, Tb: float = 0.5, top: int = 6):
    """main_setup_Couette (lbm.cpp:1537-1580) with ENERGY and D2Q9: walls
    (TYPE_S, Dirichlet TYPE_T) on rows j = 0 and Ny + 1, the top one moving
    at u_wall = Re nu / (Ny + 1), periodic in x and z; T = Tb on the fluid
    and the bottom wall, Tt = Tb + u_wall^2 / (cp Ec) on the top wall.  The
    thermal constants follow LBM.h:206-219: alpha = nu / Pr, tau_g = 0.5 +
    alpha / cs2, k = cs2 tau_g, cp = k / alpha, Ec = Br / Pr.  top: the top
    wall's type_Energy (TYPE_T, or TYPE_Q for a Neumann wall with j.n = 0).
    Returns the initialised lattice and the constants."""
    cs2 = 1.0 / 3.0
    nu = cs2 * (tau - 0.5)
    uw = Re * nu / (ny + 1)
    alpha = nu / Pr
    tau_g = 0.5 + alpha / cs2
    cp = cs2 * tau_g / alpha
    Tt = Tb + uw ** 2 / (cp * (Br / Pr))
    lat = Lattice(9, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    t[:, 0, :] = TYPE_S
    t[:, -1, :] = TYPE_S
    lat.enable_energy(tau_g, cp, nu)
    te = lat.types_energy
    te[:, 0, :] = TYPE_T
    te[:, -1, :] = top
    lat.ux[:, -1, :] = uw
    lat.T[:] = Tb
    lat.T[:, -1, :] = Tt
    lat.init()
    return lat, dict(tau=tau, tau_g=tau_g, cp=cp, nu=nu, u_wall=uw, Tb=Tb, Tt=Tt)


def rayleigh_benard(nx: int = 200, ny: int = 50, nz: int = 5):
    """main_setup_RayleighBenard1 (lbm.cpp:1585-1643) with the constants of
    LBM.h:222-242, D3Q19 with ENERGY: walls all round; the y walls Dirichlet
    (TYPE_T) at Tt on row j = 0 and Tb on row Ny + 1 (edges included), the
    x and z walls Neumann (TYPE_Q, j.n = 0) at Tt; the fluid at rest at Tt
    with F_y = g beta (T - T*), T* = (Tb + Tt) / 2, the force MacroProp
    refreshes on every cell (lbm.cpp:803-805).  Returns the initialised
    lattice and the constants."""
    cs2 = 1.0 / 3.0
    Tb, dT = 2.0, 1.0
    Tt = Tb - dT
    Ra, g_beta, Pr = 1710.0, 1e-5, 0.71
    nu = np.sqrt(g_beta * dT * float((nz + 1) ** 3) * Pr / Ra)
    tau = 0.5 + nu / cs2
    alpha = nu / Pr
    tau_g = 0.5 + alpha / cs2
    k = cs2 * tau_g
    cp = k / alpha
    T_star = (Tb + Tt) / 2
    lat = Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    lat.enable_energy(tau_g, cp, nu)
    te = lat.types_energy
    T = lat.T
    # the set-up's three ifs in order (z faces, x faces, y faces: the last
    # one wins on edges), then the y rows' temperatures
    for sl in ((0, slice(None), slice(None)), (-1, slice(None), slice(None)),
               (slice(None), slice(None), 0), (slice(None), slice(None), -1)):
        t[sl] = TYPE_S
        te[sl] = TYPE_Q
        T[sl] = Tt
    for sl in ((slice(None), 0, slice(None)), (slice(None), -1, slice(None))):
        t[sl] = TYPE_S
        te[sl] = TYPE_T
        T[sl] = Tt
    T[:, -1, :] = Tb
    T[:, 0, :] = Tt
    fl = t == TYPE_F
    T[fl] = Tt
    lat.Fy[fl] = g_beta * (Tt - T_star)
    lat.energy_buoyancy(g_beta, T_star)
    lat.init()
    return lat, dict(tau=tau, tau_g=tau_g, cp=cp, nu=nu, alpha=alpha, g_beta=g_beta, T_star=T_star, Tb=Tb, Tt=Tt)


def poiseuille(ny: int, Re: float, energy: bool = False, tau: float = 0.9, nx: int = 2, nz: int = 2):
    """main_setup_Poiseuille (lbm.cpp:1495-1535) with the constants of
    LBM.h:116-136: walls (TYPE_S; with ENERGY Dirichlet TYPE_T at Tb = Tt =
    1) on rows j = 0 and Ny + 1, periodic in x and z, u_max = Re nu /
    (Ny + 1), F_x = -dp/dx = 8 rho nu u_max / (Ny + 1)^2 on the fluid at
    set-up and, from the first MacroProp on, on every cell.  Returns the
    initialised lattice and the constants."""
    cs2 = 1.0 / 3.0
    nu = cs2 * (tau - 0.5)
    u_max = Re * nu / (ny + 1)
    fx = 8 * nu * u_max / (ny + 1) ** 2
    lat = Lattice(9, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    t[:, 0, :] = TYPE_S
    t[:, -1, :] = TYPE_S
    c = dict(tau=tau, nu=nu, u_max=u_max, fx=fx)
    if energy:
        alpha = nu / 0.7
        tau_g = 0.5 + alpha / cs2
        cp = cs2 * tau_g / alpha
        lat.enable_energy(tau_g, cp, nu)
        te = lat.types_energy
        te[:, 0, :] = TYPE_T
        te[:, -1, :] = TYPE_T
        lat.T[:] = 1.0
        c.update(tau_g=tau_g, cp=cp, alpha=alpha)
    lat.set_body_force(fx, 0.0, 0.0)
    lat.force_on_every_cell(True)
    lat.Fx[t == TYPE_F] = fx
    lat.init()
    return lat, c


def read_ref_dump(path: str, NX: int, NY: int, NZ: int, nfields: int, steps: int = 0, nodes: int = 0):
    """Read a dump written by ref_harness.cpp."""
    raw = np.fromfile(path, dtype=np.float64)
    n = NX * NY * NZ
    fields = raw[: nfields * n].reshape(nfields, NZ, NY, NX)
    rest = raw[nfields * n:]
    out = {"fields": fields}
    if steps:
        out["cl"] = rest[:steps]
        out["cd"] = rest[steps: 2 * steps]
        out["markers"] = rest[2 * steps: 2 * steps + 8 * nodes].reshape(nodes, 8)
    return out


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))


# --------------------------------------------------------------------------
# Helpers mirroring the GPU path's read-back and IBM driver
# --------------------------------------------------------------------------

def moments(lat: Lattice, body=(0.0, 0.0, 0.0), gbeta=(0.0, 0.0, 0.0), T0: float = 0.0) -> dict:
    """MacroProp moments of the post-streaming state, interior cells
    (lbm.cpp:668-679): rho = sum f, u = (sum f c + F/2) / rho with
    F = body + gbeta (T - T0); T = sum g."""
    f = lat.f[:, 1:-1, 1:-1, 1:-1]
    cx = (CX19 if lat.q == 19 else np.array([0, 1, 0, -1, 0, 1, -1, -1, 1]))
    cy = (CY19 if lat.q == 19 else np.array([0, 0, 1, 0, -1, 1, 1, -1, -1]))
    cz = (CZ19 if lat.q == 19 else np.zeros(9, int))
    rho = f.sum(axis=0)
    jx = np.tensordot(cx, f, axes=(0, 0))
    jy = np.tensordot(cy, f, axes=(0, 0))
    jz = np.tensordot(cz, f, axes=(0, 0))
    out = {"rho": rho}
    F = [np.full_like(rho, body[a]) for a in range(3)]
    if lat.thermal:
        T = lat.g[:, 1:-1, 1:-1, 1:-1].sum(axis=0)
        out["T"] = T
        for a in range(3):
            F[a] = F[a] + gbeta[a] * (T - T0)
    out["ux"] = (jx + 0.5 * F[0]) / rho
    out["uy"] = (jy + 0.5 * F[1]) / rho
    out["uz"] = (jz + 0.5 * F[2]) / rho
    return out


def internal_momentum(lat: Lattice, xc, radius: float, lo, hi) -> np.ndarray:
    out = np.zeros(6)
    c = np.ascontiguousarray(xc, dtype=np.float64)
    lo_a = (C.c_int * 3)(*lo)
    hi_a = (C.c_int * 3)(*hi)
    lib().orc_internal_momentum(lat.h, _dp(c), radius, lo_a, hi_a, _dp(out))
    return out


def body_step(body: Body, mk: Markers, radius: float, force, internal) -> None:
    f = np.ascontiguousarray(force[:6], dtype=np.float64)
    im = np.ascontiguousarray(internal[:6], dtype=np.float64)
    lib().orc_body_step(C.byref(body), C.byref(mk), radius, _dp(f), _dp(im))


def sphere_case(nx, ny, nz, tau, diameter, center, n_markers, m_max, u_in=0.05, steps=10, lit_sign=0,
                thermal=None, free=None, outlet=TYPE_OUTZG):
    """Channel + immersed sphere with the GPU path's conventions: inlet
    equilibrium at x = 0, zero-gradient outlet, bounce-back y/z walls,
    Fibonacci markers, interpolated marker density.  thermal = dict(tau_g,
    gbeta, T_in, T_body) adds the D3Q7 population and the thermal IBM;
    free = dict(rho_ratio, gravity[, dof, cv]) makes the body free (Newton-Euler;
    dof bits 0-2 translation, 3-5 rotation, default all six; cv the
    virtual-mass coefficient, default 0).
    Returns (lattice, markers, per-step force history [steps, 7], body)."""
    lat = Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = TYPE_F
    t[:, :, 0] = TYPE_IN
    t[:, :, -1] = outlet
    t[:, 0, :] = TYPE_S
    t[:, -1, :] = TYPE_S
    t[0, :, :] = TYPE_S
    t[-1, :, :] = TYPE_S
    lat.ux[t != TYPE_S] = u_in
    if thermal:
        lat.enable_thermal(thermal["tau_g"], thermal.get("T0", 0.0), thermal.get("gbeta", (0.0, 0.0, 0.0)))
        lat.T[:] = thermal.get("T_in", 0.0)
    lat.init()
    mk = fibonacci_sphere(n_markers, diameter, center)
    if thermal:
        mk["Td"][:] = thermal["T_body"]
    R = diameter / 2.0
    body = Body()
    for a in range(3):
        body.xc[a] = center[a]
    if free:
        body.rho_ratio = free["rho_ratio"]
        body.vol = np.pi * diameter ** 3 / 6.0 if "vol" not in free else free["vol"]
        body.inertia = 0.4 * body.rho_ratio * body.vol * R * R if "inertia" not in free else free["inertia"]
        for a in range(3):
            body.grav[a] = free["gravity"][a]
        body.dof = free.get("dof", 63)
        body.cv = free.get("cv", 0.0)
    hist = np.zeros((steps, 7))
    for s in range(steps):
        c = [body.xc[0], body.xc[1], body.xc[2]]
        lo, hi = sphere_box(c, diameter, lat)
        op = ibm_opts(lo, hi, m_max, lit_sign=lit_sign, rho_mode=0, thermal=1 if thermal else 0)
        out = lat.step_ibm(mk, op, c)
        hist[s] = out
        if free:
            im = internal_momentum(lat, c, R, lo, hi)
            body_step(body, mk, R, out, im)
    return lat, mk, hist, body


def read_dropin_cavity(path: str, n: int) -> dict:
    """Read the dump of the facade driver dropin_cavity (rho, ux, uy, uz, x fastest)."""
    a = np.fromfile(path, dtype=np.float64).reshape(4, n, n, n)
    return {"rho": a[0], "ux": a[1], "uy": a[2], "uz": a[3]}


# --------------------------------------------------------------------------
# MORE_DETAILS (LBM.h:55): pressure, viscous stress, running statistics
# --------------------------------------------------------------------------

# the six distinct components of a symmetric 3x3 tensor, in this order
SYM6 = ((0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2))


def details(lat: Lattice) -> dict:
    """The MORE_DETAILS part of LBM::MacroProp (lbm.cpp:681-705) over every
    cell, ghosts included, after lat.macro(): pressure = density / 3 and
    sigma[a][b] = -(tau - 0.5) * sum_l f_l (c_la - u_a)(c_lb - u_b) / tau,
    summed over l in the reference order.  sigma is returned as the six
    distinct components (SYM6 order), shape (6, NZ, NY, NX)."""
    c = (CX19, CY19, CZ19) if lat.q == 19 else (CX9, CY9, CZ9)
    u = (lat.ux, lat.uy, lat.uz)
    f = lat.f
    sig = np.empty((6,) + lat.shape)
    for s, (a, b) in enumerate(SYM6):
        acc = np.zeros(lat.shape)
        for l in range(lat.q):
            acc = acc + f[l] * (c[a][l] - u[a]) * (c[b][l] - u[b])
        sig[s] = -(lat.tau - 0.5) * acc / lat.tau
    return {"p": lat.rho / 3.0, "sigma": sig}


class SupStats:
    """The running statistics of LBM::Sup_MacroProp (lbm.cpp:865-939), FP64,
    on arrays of any shape.  update(n, ...) is the call made at reference
    step n (main.cpp:389, every nt steps) with told = (n - nt) dt.  The
    reference's own weights are kept: the velocity average weights the new
    sample by dt, every other average by 1; the pressure rms squares the
    current pressure where the other rms values square their previous rms
    (lbm.cpp:913); the Reynolds-stress rms takes u_a u_b minus the averaged
    fluctuation product.  Vorticity is never computed by the reference (its
    code is commented out, lbm.cpp:712-770), so its averages and rms stay 0
    and are not carried.  avg_rs / rms_rs hold the six distinct components
    (SYM6 order): the reference's [b][a] entries are bitwise equal to them."""

    def __init__(self, shape):
        z = lambda k: np.zeros((k,) + tuple(shape))  # noqa: E731
        self.avg_u, self.avg_p, self.avg_rs = z(3), np.zeros(shape), z(6)
        self.rms_u, self.rms_p, self.rms_rs = z(3), np.zeros(shape), z(6)

    def update(self, n: int, nt: int, dt: float, u, p) -> None:
        told = (n - nt) * dt
        for a in range(3):
            self.avg_u[a] = (self.avg_u[a] * told + u[a] * dt) / (told + dt)
        self.avg_p = (self.avg_p * told + p * 1) / (told + 1)
        d = [u[a] - self.avg_u[a] for a in range(3)]
        for s, (a, b) in enumerate(SYM6):
            self.avg_rs[s] = (self.avg_rs[s] * told + d[a] * d[b] * 1) / (told + 1)
        for a in range(3):
            self.rms_u[a] = np.sqrt((self.rms_u[a] * self.rms_u[a] * told + d[a] * d[a] * 1) / (told + 1))
        dp = p - self.avg_p
        self.rms_p = np.sqrt((p * p * told + dp * dp * 1) / (told + 1))
        for s, (a, b) in enumerate(SYM6):
            e = u[a] * u[b] - self.avg_rs[s]
            self.rms_rs[s] = np.sqrt((self.rms_rs[s] * self.rms_rs[s] * told + e * e * 1) / (told + 1))


def cavity_details_run(n: int, tau: float, lid: float, steps: int, nt: int = 10):
    """The MORE_DETAILS cavity run: Collision, Streaming, MacroProp every
    step and Sup_MacroProp every nt steps (main.cpp:214-223, 389).  Returns
    the lattice, the last details() and the statistics, ghosts included."""
    lat = cavity(n, tau, lid)
    stats = SupStats(lat.shape)
    det = None
    for s in range(1, steps + 1):
        lat.collide()
        lat.stream()
        lat.macro()
        if s % nt == 0:
            det = details(lat)
            stats.update(s, nt, 1.0, (lat.ux, lat.uy, lat.uz), det["p"])
    if det is None:
        det = details(lat)
    return lat, det, stats


def staircase2d_details_run(kind: str, nx: int, ny: int, D: float, Re: float, u_max: float, steps: int,
                            lpd: float = 1.5, nb: int = 1, nt: int = 10):
    """A staircase 2D case in MORE_DETAILS mode: Collision, Streaming,
    MacroProp every step and Sup_MacroProp every nt steps (main.cpp:214-223,
    389).  Returns the lattice, the last details() and the statistics,
    ghosts included (the reference's D2Q9 grid has three k layers)."""
    lat, boxes, area = staircase2d(kind, nx, ny, D, Re, u_max, lpd, nb)
    stats = SupStats(lat.shape)
    det = None
    for s in range(1, steps + 1):
        lat.collide()
        lat.stream()
        lat.macro()
        if s % nt == 0:
            det = details(lat)
            stats.update(s, nt, 1.0, (lat.ux, lat.uy, lat.uz), det["p"])
    if det is None:
        det = details(lat)
    return lat, det, stats


# --------------------------------------------------------------------------
# The reference's two-dimensional IBM cylinders (D2Q9)
# --------------------------------------------------------------------------

class Cylinder2D:
    """The reference's D2Q9 IBM cylinder loop (main.cpp:195-205) in its
    literal options: main_setup_Cylinder_IBM (TYPE_IN at x = 0, TYPE_OUT
    elsewhere, u = u_max), Generate_Cylinder_Marker at (Nx/5, Ny/2), and every
    step IBLBM's kinematics (lbm.cpp:1137-1167: V_CM from motion(t), markers
    and centre moved by the trapezoid, the box [floor(c - D), ceil(c + D)])
    followed by the forcing (implicit, or explicit with scheme = 1; force
    sign, nearest-node density and added mass as the reference), Collision
    and Streaming.  motion(t) -> (Vx, Vy, Vz) or None for a fixed body.
    marker_dy shifts the markers (not the centre, so not the box): the
    transverse-oscillation case generates them at center_y + amplitude
    (lbm.cpp:1966).  at_rest: the set-up of the moving-body cases
    (main_setup_Cylinder_InlineOscillating / _IBM_Moving, lbm.cpp:1878-1900,
    1980-2002): TYPE_OUT on every face, fluid at rest.  center overrides
    (Nx/5, Ny/2); area the length of C = F / (1/2 u^2 area) (D; D + dx for
    the inline oscillation, lbm.cpp:1406-1410)."""

    def __init__(self, nx: int, ny: int, D: float, nodes: int, m_max: int, u_max: float = 0.1, Re: float = 40.0,
                 scheme: int = 0, motion=None, vsolid: float | None = None, marker_dy: float = 0.0,
                 at_rest: bool = False, center=None, area: float | None = None):
        tau = 0.5 + (u_max * D / Re) / (1.0 / 3.0)
        lat = Lattice(9, nx, ny, 1, tau)
        t = lat.types
        t[:] = TYPE_F
        t[:, :, 0] = TYPE_OUT if at_rest else TYPE_IN
        t[:, :, -1] = TYPE_OUT
        t[:, 0, :] = TYPE_OUT
        t[:, -1, :] = TYPE_OUT
        lat.ux[:] = 0.0 if at_rest else u_max
        lat.init()
        self.lat, self.D, self.m_max, self.u_max, self.scheme, self.motion = lat, D, m_max, u_max, scheme, motion
        self.cx, self.cy = (nx / 5.0, ny / 2.0) if center is None else (float(center[0]), float(center[1]))
        self.area = D if area is None else area
        self.mk = cylinder_markers_literal(nodes, D, self.cx, self.cy + marker_dy)
        self.vsolid = REF_PI * D * D * 0.25 if vsolid is None else vsolid
        self.V = [0.0, 0.0, 0.0]
        self.s = 0
        self.cl, self.cd = [], []

    def step(self):
        import math

        self.s += 1
        Vold = self.V
        V = list(self.motion(self.s * 1.0)) if self.motion else [0.0, 0.0, 0.0]
        self.V = V
        mk, D = self.mk, self.D
        for a, nm in enumerate(("x", "y", "z")):
            mk[nm][:] += (V[a] + Vold[a]) * 1.0 / 2
        for a, nm in enumerate(("udx", "udy", "udz")):
            mk[nm][:] = V[a]
        self.cx += (V[0] + Vold[0]) * 1.0 / 2
        self.cy += (V[1] + Vold[1]) * 1.0 / 2
        lo = [math.floor(self.cx - D), math.floor(self.cy - D), 1]
        hi = [math.ceil(self.cx + D), math.ceil(self.cy + D), 1]
        op = ibm_opts(lo, hi, self.m_max, lit_sign=1, rho_mode=1)
        op.use_avg_density = 1
        op.vsolid = self.vsolid
        op.scheme = self.scheme
        for a in range(3):
            op.vcm_new[a] = V[a]
            op.vcm_old[a] = Vold[a]
        out = self.lat.step_ibm(mk, op, [self.cx, self.cy, 1.0])
        q = 0.5 * 1.0 * self.u_max ** 2 * self.area
        self.cl.append(out[1] / q)
        self.cd.append(out[0] / q)


def cylinder2d_literal(nx: int, ny: int, D: float, nodes: int, m_max: int, steps: int, u_max: float = 0.1,
                       Re: float = 40.0, scheme: int = 0, motion=None, vsolid: float | None = None,
                       marker_dy: float = 0.0, at_rest: bool = False, center=None, area: float | None = None):
    """Cylinder2D run for `steps` steps: the lattice, the markers, Cl and Cd
    per step (C = F / (1/2 u^2 area))."""
    c = Cylinder2D(nx, ny, D, nodes, m_max, u_max, Re, scheme, motion, vsolid, marker_dy, at_rest, center, area)
    for _ in range(steps):
        c.step()
    return c.lat, c.mk, np.array(c.cl), np.array(c.cd)


def inline_motion(u_max: float, frequency: float):
    """V_CM(t) of Cylinder_Inline_Oscillating (lbm.cpp:1142-1144)."""
    import math

    def v(t):
        return (-u_max * math.cos(2 * REF_PI * frequency * t), 0.0, 0.0)

    return v


def towed_motion(u_max: float):
    """V_CM of Cylinder_IBM_Moving_Arbie (lbm.cpp:1148-1150): -u_max along x."""

    def v(t):
        return (-u_max, 0.0, 0.0)

    return v


def transverse_motion(amplitude: float, frequency: float):
    """V_CM(t) of Cylinder_Transverse_Oscillation (lbm.cpp:1146-1148)."""
    import math

    def v(t):
        return (0.0, -2 * REF_PI * frequency * amplitude * math.sin(2 * REF_PI * frequency * t), 0.0)

    return v
