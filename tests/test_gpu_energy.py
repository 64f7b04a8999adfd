"""GPU parity for the reference's ENERGY thermal model on D2Q9 handles
(temperature populations on the flow lattice, viscous heating, Dirichlet
walls), through the C ABI: the reference's own Couette run (tests/golden)
and the FP64 oracle pinned to it.

Tolerances (FP32 arithmetic against FP64): T within 5e-3 of the run's
temperature spread max T - min T over the fluid (the viscous-heating signal),
u within 1e-5 of the wall velocity, q within 1e-5 of max |q|.  Measured: 1.2e-4 of the
spread on the reference's Couette run (u_wall = 0.0086), 2.9e-3 on the
forced case (u_wall = 0.12, 777 steps).  The second is FP32 rounding of the
stored populations, biased alike every step in a steady flow: a float64
restatement of the same pull algorithm agrees with the oracle to 1e-11, a
float32 one differs from it by 1.2e-6 in T, as the kernel does (1.8e-6)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _couette_setup(orc, ny, Re, nx=2, tau=0.9, u_bottom=0.0, Tb=0.5, top=None, bottom=None):
    """The arrays of main_setup_Couette's k = 1 layer (lbm.cpp:1537-1580)
    and the LBM.h constants; top / bottom: the walls' type_Energy (TYPE_T
    by default)."""
    cs2 = 1.0 / 3.0
    nu = cs2 * (tau - 0.5)
    uw = Re * nu / (ny + 1)
    Pr, Br = 0.7, 10.0
    alpha = nu / Pr
    tau_g = 0.5 + alpha / cs2
    cp = cs2 * tau_g / alpha
    Tt = Tb + uw ** 2 / (cp * (Br / Pr))
    t = np.zeros((ny + 2, nx + 2), np.uint8)
    t[0, :] = orc.TYPE_S
    t[-1, :] = orc.TYPE_S
    te = np.zeros_like(t)
    te[0, :] = orc.TYPE_T if bottom is None else bottom
    te[-1, :] = orc.TYPE_T if top is None else top
    ux = np.zeros(t.shape)
    ux[-1, :] = uw
    ux[0, :] = u_bottom
    T = np.full(t.shape, Tb)
    T[-1, :] = Tt
    return t, te, ux, T, dict(tau=tau, tau_g=tau_g, cp=cp, nu=nu, u_wall=uw, Tb=Tb, Tt=Tt)


def _solver(pkg, orc, ny, Re, storage="f32", graph_steps=0, body=0.0, **kw):
    t, te, ux, T, c = _couette_setup(orc, ny, Re, **kw)
    nx = t.shape[1] - 2
    cfg = pkg.config_from_types_2d(nx, ny, c["tau"], t, np.ones(t.shape), ux, np.zeros(t.shape))
    cfg = pkg.config_energy_2d(cfg, nx, ny, t, te, T, c["tau_g"], c["cp"])
    assert cfg.thermal == pkg.THERMAL_ENERGY and (cfg.nx, cfg.ny) == (nx + 2, ny)
    cfg.storage = pkg.STORAGE[storage]
    cfg.graph_steps = graph_steps
    cfg.body_force[0] = body
    s = pkg.Solver(cfg)
    s.init()
    return s, c


def _check(s, pkg, T, u, q, uref, tol_T=5e-3):
    m = s.moments()
    spread = T.max() - T.min()
    eT = np.abs(m["T"][0] - T).max() / spread
    eu = max(np.abs(m["ux"][0] - u[0]).max(), np.abs(m["uy"][0] - u[1]).max()) / uref
    qx = s.download_f32(pkg.FIELD_QX)[0]
    qy = s.download_f32(pkg.FIELD_QY)[0]
    eq = max(np.abs(qx - q[0]).max(), np.abs(qy - q[1]).max()) / np.abs(q).max()
    assert eT < tol_T and eu < 1e-5 and eq < 1e-5, (eT, eu, eq)
    assert not np.any(m["uz"]) and not np.any(s.download_f32(pkg.FIELD_QZ))
    return eT, eu, eq


def test_energy_couette_vs_reference(pkg, orc):
    """The reference's own run: 2000 steps, every fluid row (the periodic
    ghost columns included)."""
    g = np.load(os.path.join(GOLDEN, "couette_energy_ny30_re20_2000.npz"))
    s, c = _solver(pkg, orc, int(g["ny"]), float(g["Re"]))
    s.step(int(g["steps"]))
    assert s.status() == 0
    e = _check(s, pkg, g["T"][1:-1], g["u"][:2, 1:-1], g["q"][:2, 1:-1], c["u_wall"])
    print("couette T / u / q errors: %.3g %.3g %.3g" % e)
    # viscous heating: the centre is warmer than both walls
    T = s.moments()["T"][0]
    assert T[T.shape[0] // 2].mean() > T[0].mean() + 1e-4


def test_energy_forced_moving_walls_vs_oracle(pkg, orc):
    """Both walls moving, a body force, a wider periodic channel, an odd step
    count (the graphs' remainder path)."""
    ny, Re, steps, fx = 24, 30.0, 777, 1e-6
    s, c = _solver(pkg, orc, ny, Re, nx=6, u_bottom=-0.01, body=fx, tau=0.8)
    s.step(steps)
    assert s.status() == 0
    lat, _ = orc.couette_energy(ny, Re, tau=0.8, nx=6)
    lat.ux[:, 0, :] = -0.01
    lat.init()
    lat.set_body_force(fx, 0.0, 0.0)
    lat.Fx[lat.types == orc.TYPE_F] = fx
    assert lat.step_plain(steps) == 0
    L = slice(1, -1)
    e = _check(s, pkg, lat.T[1, L], np.stack([lat.ux[1, L], lat.uy[1, L]]), lat.hq[:2, 1, L], c["u_wall"])
    print("forced T / u / q errors: %.3g %.3g %.3g" % e)


def test_energy_couette_neumann_vs_reference(pkg, orc):
    """The top wall a Neumann wall (type_Energy TYPE_Q, j.n = 0): its T from
    the cell's g in the middle of the reference's push, whose result depends
    on the visiting order (Determine_Twall_Neumann, lbm.cpp:983-1028).
    Against the reference's own single-thread run, 1000 steps, every fluid
    row."""
    g = np.load(os.path.join(GOLDEN, "couette_neumann_ny30_re20_1000.npz"))
    s, c = _solver(pkg, orc, int(g["ny"]), float(g["Re"]), top=orc.TYPE_Q)
    s.step(int(g["steps"]))
    assert s.status() == 0
    e = _check(s, pkg, g["T"][1:-1], g["u"][:2, 1:-1], g["q"][:2, 1:-1], c["u_wall"])
    print("couette Neumann T / u / q errors: %.3g %.3g %.3g" % e)
    # no heat crosses the top wall: the profile flattens towards it
    T = s.moments()["T"][0][:, 1]
    assert abs(T[-1] - T[-2]) < 0.1 * abs(T[1] - T[0])


@pytest.mark.parametrize("case", ["neumann_bottom", "adiabatic_top"])
def test_energy_neumann_adiabatic_vs_oracle(pkg, orc, case):
    """A Neumann bottom wall under a moving Dirichlet top (the links from
    above come from cells the reference's push visits later: last sweep's
    values), and an adiabatic top wall (type_Energy TYPE_F: its links keep
    their initial values); a wider channel, a moving bottom wall, an odd
    step count."""
    ny, Re, steps, nx, tau = 24, 30.0, 555, 6, 0.8
    kw = dict(bottom=orc.TYPE_Q) if case == "neumann_bottom" else dict(top=orc.TYPE_F)
    s, c = _solver(pkg, orc, ny, Re, nx=nx, u_bottom=-0.01, tau=tau, **kw)
    s.step(steps)
    assert s.status() == 0
    lat, _ = orc.couette_energy(ny, Re, tau=tau, nx=nx, top=kw.get("top", orc.TYPE_T))
    lat.ux[:, 0, :] = -0.01
    if "bottom" in kw:
        lat.types_energy[:, 0, :] = kw["bottom"]
    lat.init()
    assert lat.step_plain(steps) == 0
    L = slice(1, -1)
    e = _check(s, pkg, lat.T[1, L], np.stack([lat.ux[1, L], lat.uy[1, L]]), lat.hq[:2, 1, L], c["u_wall"])
    print("%s T / u / q errors: %.3g %.3g %.3g" % ((case,) + e))


@pytest.mark.parametrize("top", ["dirichlet", "neumann"])
def test_energy_graph_replay_matches_eager(pkg, orc, top):
    out = []
    for gs in (8, -1):
        s, _ = _solver(pkg, orc, 30, 20.0, graph_steps=gs, top=orc.TYPE_Q if top == "neumann" else None)
        s.step(203)
        m = s.moments()
        out.append((m["T"], m["ux"], s.download_f32(pkg.FIELD_QY)))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_energy_unsupported_calls_fail_loudly(pkg, orc):
    s, c = _solver(pkg, orc, 10, 20.0)
    with pytest.raises(pkg.LbmError) as e:
        s.set_markers(np.zeros((3, 4)), np.ones(4), 1.0, (2.0, 5.0, 1.0))
    assert e.value.status == 7
    # half storage: geq = rho w T makes T integrate every error of rho
    for st in ("f16", "bf16"):
        with pytest.raises(pkg.LbmError) as e:
            _solver(pkg, orc, 10, 20.0, storage=st)
        assert e.value.status == 7 and "FP32" in str(e.value)


@pytest.mark.parametrize("energy", [False, True], ids=["plain", "energy"])
def test_poiseuille_wall_force_vs_reference(pkg, orc, energy):
    """The reference's Poiseuille_Flow build: F = -dp/dx on every cell in
    MacroProp, so its walls move at F/2 from the third streaming on
    (lbm_config.wall_force); with ENERGY the walls at T = 1 and viscous
    heating.  Against the reference's own 1500-step runs."""
    g = np.load(os.path.join(GOLDEN, "poiseuille_ny30_re20%s_1500.npz" % ("_energy" if energy else "")))
    ny, Re = int(g["ny"]), float(g["Re"])
    lat, c = orc.poiseuille(ny, Re, energy=energy)
    t = lat.types[1].copy()
    nx = t.shape[1] - 2
    cfg = pkg.config_from_types_2d(nx, ny, c["tau"], t, np.ones(t.shape), np.zeros(t.shape), np.zeros(t.shape))
    if energy:
        te = np.zeros_like(t)
        te[0, :] = te[-1, :] = orc.TYPE_T
        cfg = pkg.config_energy_2d(cfg, nx, ny, t, te, np.ones(t.shape), c["tau_g"], c["cp"])
    cfg.body_force[0] = c["fx"]
    cfg.wall_force = 1
    s = pkg.Solver(cfg)
    s.init()
    s.step(int(g["steps"]))
    assert s.status() == 0
    m = s.moments()
    um = np.abs(g["u"][0, 1:-1]).max()
    eu = max(np.abs(m["ux"][0] - g["u"][0, 1:-1]).max(), np.abs(m["uy"][0] - g["u"][1, 1:-1]).max()) / um
    print("poiseuille %s u error / u_max: %.3g" % ("energy" if energy else "plain", eu))
    # FP32 over 1500 steps: measured 1.3e-5; a run without the walls' drift
    # is off by 5.5e-4 (checked below)
    assert eu < 3e-5
    if energy:
        T = g["T"][1:-1]
        eT = np.abs(m["T"][0] - T).max() / (T.max() - T.min())
        print("poiseuille T error / spread: %.3g" % eT)
        assert eT < 5e-3
    # without the walls' drift the profile differs by about the wall speed F/2
    cfg.wall_force = 0
    s2 = pkg.Solver(cfg)
    s2.init()
    s2.step(int(g["steps"]))
    assert np.abs(s2.moments()["ux"][0] - g["u"][0, 1:-1]).max() > 0.3 * 0.5 * c["fx"]
