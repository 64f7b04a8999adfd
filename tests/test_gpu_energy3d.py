"""The reference's ENERGY model on D3Q19 (lbm_energy3d): its Rayleigh_Benard
case (main_setup_RayleighBenard1, lbm.cpp:1585-1643; LBM.h:222-242) against
the reference's own single-thread run and, at the case's own 200 x 50 x 5
size, against the FP64 oracle; a lid-driven box with a periodic axis,
adiabatic and Neumann walls against the oracle.

Fields are FP32 against FP64.  T starts at Tt = 1 in the fluid with the
walls at 1 and 2; its error stays at the FP32 rounding of T ~ 1-2 integrated
over the steps (measured 2.1e-6 of the temperature spread after 400 steps,
1.7e-6 at full size after 200), the velocity (at most 1e-4 here, driven by
the buoyancy g beta = 1e-5) within 1.3e-5 of its largest value, which is
the FP32 rounding of the momentum sums near rho = 1 (6e-8) against
|u| ~ 1e-4 over a few hundred steps.  The bounds leave a factor of 5 to 10."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _rb_gpu(pkg, lat, c, graph_steps=0):
    """The GPU solver on the oracle lattice's set-up arrays (the oracle's
    restatement of main_setup_RayleighBenard1, before any step)."""
    return pkg.Energy3D(lat.types.copy(), lat.types_energy.copy(), lat.T.copy(), c["tau"], c["tau_g"], c["cp"],
                        g_beta=c["g_beta"], T_star=c["T_star"], F=np.stack([lat.Fx, lat.Fy, lat.Fz]).copy(),
                        graph_steps=graph_steps)


def _errors(m, ref, fluid):
    spread = ref["T"][fluid].max() - ref["T"][fluid].min()
    eT = np.abs(m["T"][fluid] - ref["T"][fluid]).max() / spread
    us = max(np.abs(ref[k][fluid]).max() for k in ("ux", "uy", "uz"))
    eu = max(np.abs(m[k][fluid] - ref[k][fluid]).max() for k in ("ux", "uy", "uz")) / us
    er = np.abs(m["rho"][fluid] - ref["rho"][fluid]).max()
    qs = max(np.abs(ref[k][fluid]).max() for k in ("qx", "qy", "qz"))
    eq = max(np.abs(m[k][fluid] - ref[k][fluid]).max() for k in ("qx", "qy", "qz")) / qs
    return eT, eu, er, eq


def test_rayleigh_benard_vs_reference(pkg, orc):
    """The reference's run on one thread (its Neumann walls make the result
    depend on the visiting order), 400 steps on a 32 x 16 x 5 box, every
    fluid cell."""
    g = np.load(os.path.join(GOLDEN, "rayleigh32x16x5_400.npz"))
    lat, c = orc.rayleigh_benard(int(g["nx"]), int(g["ny"]), int(g["nz"]))
    s = _rb_gpu(pkg, lat, c)
    s.step(int(g["steps"]))
    assert s.status() == 0
    m = s.moments()
    fluid = lat.types == orc.TYPE_F
    ref = dict(rho=g["rho"], ux=g["u"][0], uy=g["u"][1], uz=g["u"][2], T=g["T"], qx=g["q"][0], qy=g["q"][1],
               qz=g["q"][2])
    eT, eu, er, eq = _errors(m, ref, fluid)
    print("rayleigh 32x16x5, 400 steps: T %.3g of spread, u %.3g of max, rho %.3g, q %.3g of max" % (eT, eu, er, eq))
    assert eT < 1e-5 and eu < 1e-4 and er < 1e-6 and eq < 1e-4, (eT, eu, er, eq)
    # the walls: MacroProp's sums of their initial populations, moving at
    # F / (2 rho) (host values in FP64)
    for k in ref:
        assert np.allclose(m[k][~fluid], ref[k][~fluid], rtol=1e-12, atol=1e-18), k


def test_rayleigh_benard_fullsize_vs_oracle(pkg, orc):
    """The case at its own size (200 x 50 x 5), 200 steps, against the oracle
    (bit-exact with the reference on the smaller box), with the maximum
    vertical velocity and the Nusselt number of its main loop
    (Find_Maximum_uy, Find_Nusselt_number, main.cpp:308-321)."""
    steps = 200
    lat, c = orc.rayleigh_benard(200, 50, 5)
    s = _rb_gpu(pkg, lat, c)
    s.step(steps)
    assert s.status() == 0
    m = s.moments()
    assert lat.step_plain(steps) == 0
    fluid = lat.types == orc.TYPE_F
    ref = dict(rho=lat.rho, ux=lat.ux, uy=lat.uy, uz=lat.uz, T=lat.T, qx=lat.hq[0], qy=lat.hq[1], qz=lat.hq[2])
    eT, eu, er, eq = _errors(m, ref, fluid)
    uy_g, uy_o = np.abs(m["uy"][fluid]).max(), np.abs(lat.uy[fluid]).max()
    # Find_Nusselt_number: 1 + <uy T> / (alpha dT / H) over the fluid cells
    H = 50 + 1
    nu_g = 1 + (m["uy"][fluid] * m["T"][fluid]).mean() / (c["alpha"] * 1.0 / H)
    nu_o = 1 + (lat.uy[fluid] * lat.T[fluid]).mean() / (c["alpha"] * 1.0 / H)
    print("rayleigh 200x50x5, %d steps: T %.3g of spread, u %.3g of max, rho %.3g, q %.3g; max|uy| %.6g / %.6g, "
          "Nu %.8f / %.8f" % (steps, eT, eu, er, eq, uy_g, uy_o, nu_g, nu_o))
    assert eT < 1e-5 and eu < 1e-4 and er < 1e-6 and eq < 1e-4, (eT, eu, er, eq)
    # Nu - 1 carries the relative error of uy (measured 9.4e-6 of Nu - 1)
    assert abs(uy_g - uy_o) < 1e-4 * uy_o and abs(nu_g - nu_o) < 1e-4 * abs(nu_o - 1.0)


def test_rayleigh_benard_larger_box_vs_oracle(pkg, orc):
    """The same set-up on a 128 x 64 x 32 box, where the wall records are
    under an eighth of the grid and the Neumann pre-pass runs one thread a
    record (the warp-a-record form serves the smaller boxes above); 60 steps
    against the oracle."""
    steps = 60
    lat, c = orc.rayleigh_benard(128, 64, 32)
    s = _rb_gpu(pkg, lat, c)
    s.step(steps)
    assert s.status() == 0
    m = s.moments()
    assert lat.step_plain(steps) == 0
    fluid = lat.types == orc.TYPE_F
    ref = dict(rho=lat.rho, ux=lat.ux, uy=lat.uy, uz=lat.uz, T=lat.T, qx=lat.hq[0], qy=lat.hq[1], qz=lat.hq[2])
    eT, eu, er, eq = _errors(m, ref, fluid)
    print("rayleigh 128x64x32, %d steps: T %.3g of spread, u %.3g of max, rho %.3g, q %.3g" % (steps, eT, eu, er, eq))
    assert eT < 1e-5 and eu < 1e-4 and er < 1e-6 and eq < 1e-4, (eT, eu, er, eq)


def test_lid_box_periodic_adiabatic_vs_oracle(pkg, orc):
    """A box with a moving lid (the y+ wall, u_x = 0.05, Dirichlet at T = 1.2),
    a Dirichlet floor at 1, Neumann x walls, an adiabatic wall
    (type_Energy TYPE_F) at x = 0 above mid-height, and fluid ghost layers
    in z (the reference's periodic modulo over the whole grid); buoyancy on.
    333 steps against the oracle."""
    nx, ny, nz, steps = 20, 14, 6, 333
    tau, Pr = 0.7, 0.71
    cs2 = 1.0 / 3.0
    nu = cs2 * (tau - 0.5)
    alpha = nu / Pr
    tau_g = 0.5 + alpha / cs2
    cp = cs2 * tau_g / alpha
    lat = orc.Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = orc.TYPE_F
    lat.enable_energy(tau_g, cp, nu)
    te = lat.types_energy
    T = lat.T
    for sl in ((slice(None), slice(None), 0), (slice(None), slice(None), -1)):
        t[sl] = orc.TYPE_S
        te[sl] = orc.TYPE_Q
    t[:, 0, :] = orc.TYPE_S
    te[:, 0, :] = orc.TYPE_T
    t[:, -1, :] = orc.TYPE_S
    te[:, -1, :] = orc.TYPE_T
    te[:, ny // 2:, 0] = orc.TYPE_F
    T[:] = 1.0
    T[:, -1, :] = 1.2
    lat.ux[:, -1, :] = 0.05
    fl = t == orc.TYPE_F
    lat.Fy[fl] = 1e-5 * (1.0 - 1.1)
    lat.energy_buoyancy(1e-5, 1.1)
    s = pkg.Energy3D(t.copy(), te.copy(), T.copy(), tau, tau_g, cp, g_beta=1e-5, T_star=1.1,
                     u=np.stack([lat.ux, lat.uy, lat.uz]).copy(), F=np.stack([lat.Fx, lat.Fy, lat.Fz]).copy())
    lat.init()
    s.step(steps)
    assert s.status() == 0
    m = s.moments()
    assert lat.step_plain(steps) == 0
    ref = dict(rho=lat.rho, ux=lat.ux, uy=lat.uy, uz=lat.uz, T=lat.T, qx=lat.hq[0], qy=lat.hq[1], qz=lat.hq[2])
    eT, eu, er, eq = _errors(m, ref, fl)
    print("lid box 20x14x6, %d steps: T %.3g of spread, u %.3g of max, rho %.3g, q %.3g" % (steps, eT, eu, er, eq))
    # measured T 1.9e-6, u 6.6e-7, rho 6.3e-8, q 1.5e-6
    assert eT < 2e-5 and eu < 1e-5 and er < 1e-6 and eq < 2e-5, (eT, eu, er, eq)


def test_moving_interior_solid_vs_oracle(pkg, orc):
    """A 2 x 2 x 2 solid block inside the fluid, moving with u_x = 0.02
    (Determine_Wall_Velocity's moving solid neighbours, lbm.cpp:941-962) and
    held at T = 1.1 (type_Energy TYPE_T), in a channel with Dirichlet y walls
    and fluid ghost layers in x and z (the periodic modulo over the whole
    grid); 250 steps against the oracle."""
    nx, ny, nz, steps, tau = 16, 12, 8, 250, 0.75
    cs2 = 1.0 / 3.0
    nu = cs2 * (tau - 0.5)
    alpha = nu / 0.71
    tau_g = 0.5 + alpha / cs2
    cp = cs2 * tau_g / alpha
    lat = orc.Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = orc.TYPE_F
    lat.enable_energy(tau_g, cp, nu)
    te = lat.types_energy
    T = lat.T
    T[:] = 1.0
    t[:, 0, :] = t[:, -1, :] = orc.TYPE_S
    te[:, 0, :] = te[:, -1, :] = orc.TYPE_T
    blk = (slice(4, 6), slice(5, 7), slice(7, 9))  # k, j, i
    t[blk] = orc.TYPE_S
    te[blk] = orc.TYPE_T
    T[blk] = 1.1
    lat.ux[blk] = 0.02
    s = pkg.Energy3D(t.copy(), te.copy(), T.copy(), tau, tau_g, cp, u=np.stack([lat.ux, lat.uy, lat.uz]).copy())
    lat.init()
    s.step(steps)
    assert s.status() == 0
    m = s.moments()
    assert lat.step_plain(steps) == 0
    fl = t == orc.TYPE_F
    ref = dict(rho=lat.rho, ux=lat.ux, uy=lat.uy, uz=lat.uz, T=lat.T, qx=lat.hq[0], qy=lat.hq[1], qz=lat.hq[2])
    eT, eu, er, eq = _errors(m, ref, fl)
    print("moving block 16x12x8, %d steps: T %.3g of spread, u %.3g of max, rho %.3g, q %.3g" % (steps, eT, eu, er, eq))
    assert eT < 2e-5 and eu < 1e-5 and er < 1e-6 and eq < 2e-5, (eT, eu, er, eq)
    # the block drags the fluid along x
    assert m["ux"][fl].max() > 1e-3


@pytest.mark.parametrize("graph_steps", [0, 3])
def test_energy3d_graph_replay_matches_eager(pkg, orc, graph_steps):
    """Steps replayed from captured graphs (the default ten, and an odd
    request rounded up to four), between eager ones and across both starting
    buffers, give the same bits as every step launched on its own."""
    lat, c = orc.rayleigh_benard(200, 50, 5)
    out = []
    for gs in (graph_steps, -1):
        s = _rb_gpu(pkg, lat, c, graph_steps=gs)
        for n in (2, 11, 1, 24, 5):
            s.step(n)
        assert s.status() == 0
        out.append(s.moments())
    for k in out[1]:
        assert np.array_equal(out[0][k], out[1][k], equal_nan=True), k


def test_energy3d_rejects_other_cell_types(pkg, orc):
    lat, c = orc.rayleigh_benard(8, 6, 4)
    t = lat.types.copy()
    t[2, 2, 2] = orc.TYPE_IN
    with pytest.raises(pkg.LbmError) as e:
        pkg.Energy3D(t, lat.types_energy.copy(), lat.T.copy(), c["tau"], c["tau_g"], c["cp"])
    assert e.value.status == 7
