"""GPU parity for interior solid cells (staircase bodies): halfway bounce-back
on the links of solid cells inside the fused step, and the momentum exchange
on them (MEA_CD / MEA_CL, lbm.cpp:3085-3163), against the reference's own
Sphere_BB run (tests/golden) and the FP64 oracle.

Tolerances: FP32 fields within 1e-5 of the inflow velocity U, Cd / Cl within
1e-4 of the largest |Cd| of the run; FP16 storage drag within 0.5 %."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

PI_REF = 3.14159265


def _sphere_solver(pkg, orc, nx, ny, nz, tau, D, u, storage="f32", graph_steps=0):
    lat, box = orc.sphere_bb(nx, ny, nz, tau, D, u)
    cfg = pkg.config_from_types(nx, ny, nz, tau, lat.types.copy(), lat.rho.copy(), lat.ux.copy(), lat.uy.copy(),
                                lat.uz.copy())
    cfg.storage = pkg.STORAGE[storage]
    cfg.graph_steps = graph_steps
    s = pkg.Solver(cfg)
    s.set_solids(lat.interior(lat.types) == orc.TYPE_S)
    s.init([lat.interior(getattr(lat, c)) for c in ("rho", "ux", "uy", "uz")])
    return s, lat, box


def _coeffs(rows, u, D):
    area = 0.5 * u * u * D * D * PI_REF / 4.0
    return rows[:, 0] / area, -rows[:, 1] / area


def test_staircase_sphere_vs_reference_golden(pkg, orc):
    g = np.load(os.path.join(GOLDEN, "sphere_bb48x24x24_D8_Re20_100.npz"))
    nx, ny, nz, D, Re, u = int(g["nx"]), int(g["ny"]), int(g["nz"]), float(g["D"]), float(g["Re"]), float(g["u"])
    steps = int(g["steps"])
    tau = 0.5 + (u * D / Re) / (1.0 / 3.0)
    s, _, _ = _sphere_solver(pkg, orc, nx, ny, nz, tau, D, u)
    s.step(steps)
    assert s.status() == 0
    m = s.moments()
    f = np.stack([m[c] for c in ("rho", "ux", "uy", "uz")])
    eu = max(np.abs(f[1:, 12] - g["zmid"][1:]).max(), np.abs(f[1:, :, 12] - g["ymid"][1:]).max()) / u
    er = max(np.abs(f[0, 12] - g["zmid"][0]).max(), np.abs(f[0, :, 12] - g["ymid"][0]).max())
    assert eu < 1e-5 and er < 1e-5, (eu, er)
    rows = s.solid_forces()
    assert rows.shape[0] == steps
    assert np.array_equal(rows[:, 3], np.arange(1, steps + 1))
    cd, cl = _coeffs(rows, u, D)
    scale = np.abs(g["cd"]).max()
    assert np.abs(cd - g["cd"]).max() / scale < 1e-4, np.abs(cd - g["cd"]).max() / scale
    assert np.abs(cl - g["cl"]).max() / scale < 1e-4, np.abs(cl - g["cl"]).max() / scale


def test_staircase_sphere_fp16_drag(pkg, orc):
    nx, ny, nz, D, u, steps = 48, 24, 24, 8.0, 0.05, 150
    tau = 0.56
    s, lat, box = _sphere_solver(pkg, orc, nx, ny, nz, tau, D, u, storage="f16")
    s.step(steps)
    assert s.status() == 0
    cd, _ = _coeffs(s.solid_forces(), u, D)
    area = 0.5 * u * u * D * D * PI_REF / 4.0
    ref = []
    for _ in range(steps):
        lat.collide()
        lat.stream()
        lat.macro()
        ref.append(-lat.mea(box)[0] / area)
    ref = np.array(ref)
    assert abs(cd[-1] - ref[-1]) / abs(ref[-1]) < 5e-3, (cd[-1], ref[-1])
    m = s.moments()
    assert np.abs(m["ux"] - lat.interior(lat.ux)).max() / u < 2e-3


def test_staircase_cylinder_periodic_z_vs_oracle(pkg, orc):
    """A staircase cylinder across a channel that is periodic in z (TYPE_F
    ghost planes), bounce-back walls in y: solid links across the periodic
    seam and next to the walls."""
    nx, ny, nz, tau, u, steps = 40, 20, 6, 0.6, 0.04, 120
    lat = orc.Lattice(19, nx, ny, nz, tau)
    t = lat.types
    t[:] = orc.TYPE_F
    t[:, :, 0] = orc.TYPE_IN
    t[:, :, -1] = orc.TYPE_OUT
    t[:, 0, :] = orc.TYPE_S
    t[:, -1, :] = orc.TYPE_S
    k, j, i = np.meshgrid(np.arange(nz + 2), np.arange(ny + 2), np.arange(nx + 2), indexing="ij")
    # the body spans the interior planes; the periodic ghost planes, which the
    # device also holds, stay fluid
    body = ((i - 10.5) ** 2 + (j - 9.0) ** 2 <= 3.2 ** 2) & (i >= 1) & (i <= nx) & (j >= 1) & (j <= ny) & \
        (k >= 1) & (k <= nz)
    t[body] = orc.TYPE_S
    lat.ux[(t != orc.TYPE_S)] = u
    lat.init()
    cfg = pkg.config_from_types(nx, ny, nz, tau, t.copy(), lat.rho.copy(), lat.ux.copy(), lat.uy.copy(),
                                lat.uz.copy())
    s = pkg.Solver(cfg)
    # the periodic z axis spans all N+2 planes on the device (the reference
    # wraps over its ghost planes too)
    s.set_solids(body[:, 1:-1, 1:-1])
    s.init([getattr(lat, c)[:, 1:-1, 1:-1] for c in ("rho", "ux", "uy", "uz")])
    s.step(steps)
    assert s.status() == 0
    lat.step_plain(steps)
    m = s.moments()
    f = lat.f[:, :, 1:-1, 1:-1]
    rho = f.sum(axis=0)
    from oracle import CX19, CY19

    ux = np.tensordot(CX19, f, axes=(0, 0)) / rho
    uy = np.tensordot(CY19, f, axes=(0, 0)) / rho
    solid = body[:, 1:-1, 1:-1]
    fl = ~solid
    assert np.abs(m["ux"][fl] - ux[fl]).max() / u < 1e-5
    assert np.abs(m["uy"][fl] - uy[fl]).max() / u < 1e-5
    assert np.abs(m["rho"][fl] - rho[fl]).max() < 1e-5
    assert np.allclose(m["rho"][solid], 1.0, atol=1e-6) and np.abs(m["ux"][solid]).max() < 1e-7


def test_graph_replay_matches_eager_with_solids(pkg, orc):
    out = []
    for gs in (10, 0):
        s, _, _ = _sphere_solver(pkg, orc, 48, 24, 24, 0.56, 8.0, 0.05, graph_steps=gs)
        for n in (1, 10, 3, 20):
            s.step(n)
        out.append((s.moments(), s.solid_forces()))
    for c in out[0][0]:
        assert np.array_equal(out[0][0][c], out[1][0][c]), c
    assert np.array_equal(out[0][1], out[1][1])


def test_set_solids_after_init_is_refused(pkg, orc):
    s, lat, _ = _sphere_solver(pkg, orc, 48, 24, 24, 0.56, 8.0, 0.05)
    with pytest.raises(pkg.LbmError) as e:
        s.set_solids(lat.interior(lat.types) == orc.TYPE_S)
    assert e.value.status == 6
