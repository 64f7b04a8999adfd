"""GPU parity: the fused collide-stream kernel through the C ABI against the
FP64 oracle and the reference's own golden output (lid-driven cavity).

Tolerance: plain FP32 fields within 1e-5 of the lid velocity U, also on the
64^3, 5000-step cavity against the reference's own FP64 run (measured there:
3.1e-6 U, max over the mid planes).  FP16/BF16 shifted-population storage
errors are measured and bounded (FP16 1.5e-3 U, BF16 2e-2 U)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-5


def _err(m, ref, lid):
    eu = max(np.abs(m[c] - ref[c]).max() for c in ("ux", "uy", "uz")) / lid
    er = np.abs(m["rho"] - ref["rho"]).max()
    return eu, er


@pytest.mark.parametrize("cells", [1, 2])
@pytest.mark.parametrize("shape,tau", [((16, 16, 16), 0.8), ((12, 18, 10), 0.6), ((33, 20, 17), 0.55),
                                       ((64, 9, 7), 0.7)])
def test_cavity_fp32_vs_oracle(pkg, orc, shape, tau, cells):
    """One and two cells per thread (a row of 33 cells takes one either
    way)."""
    nx, ny, nz = shape
    lid, steps = 0.05, 300
    s = pkg.Solver(pkg.cavity_config(nx, tau=tau, lid=lid, ny=ny, nz=nz, cells=cells))
    s.init()
    s.step(steps)
    m = s.moments()
    assert s.status() == 0
    lat = orc.cavity(nx, tau, lid, ny=ny, nz=nz)
    lat.step_plain(steps)
    eu, er = _err(m, orc.moments(lat), lid)
    assert eu < TOL_F32 and er < TOL_F32, (eu, er)


def test_cavity64_5000_vs_reference_golden(pkg):
    """The 64^3, tau = 0.8, 5000-step cavity against the reference's own run."""
    g = np.load(os.path.join(GOLDEN, "cavity64_tau0.8_lid0.05_5000.npz"))
    lid = float(g["lid"])
    res = {}
    for st in ("f32", "f16", "bf16"):
        s = pkg.Solver(pkg.cavity_config(64, tau=0.8, lid=lid, storage=st))
        s.init()
        s.step(int(g["steps"]))
        m = s.moments()
        assert s.status() == 0
        f = np.stack([m["rho"], m["ux"], m["uy"], m["uz"]])
        ez = np.abs(f[:, 32] - g["zmid"]).max(axis=(1, 2))
        ex = np.abs(f[:, :, :, 32] - g["xmid"]).max(axis=(1, 2))
        e = np.maximum(ez, ex)
        res[st] = (e[0], e[1:].max() / lid)
        s.close()
    print("cavity64 errors (rho abs, u / U):", res)
    assert res["f32"][0] < TOL_F32 and res["f32"][1] < TOL_F32
    assert res["f16"][1] < 1.5e-3
    assert res["bf16"][1] < 2e-2


def test_graph_replay_matches_eager_bitwise(pkg):
    a = pkg.Solver(pkg.cavity_config(24, tau=0.7, lid=0.04, graph_steps=8))
    b = pkg.Solver(pkg.cavity_config(24, tau=0.7, lid=0.04, graph_steps=-1))
    for s in (a, b):
        s.init()
        s.step(1)
        s.step(37)
        s.step(20)
    ma, mb = a.moments(), b.moments()
    for c in ("rho", "ux", "uy", "uz"):
        assert np.array_equal(ma[c], mb[c]), c


def test_download_before_first_step_is_initial_state(pkg):
    s = pkg.Solver(pkg.cavity_config(8, tau=0.8, lid=0.05, u0=(0.01, 0.0, 0.0)))
    s.init()
    m = s.moments()
    assert np.allclose(m["rho"], 1.0, atol=1e-6)
    assert np.allclose(m["ux"], 0.01, atol=1e-7)


def test_init_fields_matches_oracle_nonuniform(pkg, orc):
    n, tau, lid, steps = 12, 0.7, 0.05, 120
    rng = np.random.default_rng(7)
    rho = 1.0 + 0.01 * rng.standard_normal((n, n, n))
    ux = 0.01 * rng.standard_normal((n, n, n))
    uy = 0.01 * rng.standard_normal((n, n, n))
    uz = 0.01 * rng.standard_normal((n, n, n))
    s = pkg.Solver(pkg.cavity_config(n, tau=tau, lid=lid))
    s.init((rho, ux, uy, uz))
    s.step(steps)
    m = s.moments()
    lat = orc.Lattice(19, n, n, n, tau)
    t = lat.types
    t[:] = orc.TYPE_S
    t[1:-1, 1:-1, 1:-1] = orc.TYPE_F
    lat.ux[:, -1, :] = lid
    lat.rho[1:-1, 1:-1, 1:-1] = rho
    lat.ux[1:-1, 1:-1, 1:-1] = ux
    lat.uy[1:-1, 1:-1, 1:-1] = uy
    lat.uz[1:-1, 1:-1, 1:-1] = uz
    lat.init()
    lat.step_plain(steps)
    eu, er = _err(m, orc.moments(lat), lid)
    assert eu < TOL_F32 and er < TOL_F32, (eu, er)


def test_status_flags_invalid_density(pkg):
    """A NaN initial density (a host-side fault) is reported by the device
    status word and the ABI's status code, never by a trap."""
    n = 8
    rho = np.ones((n, n, n))
    rho[3, 3, 3] = np.nan
    z = np.zeros((n, n, n))
    s = pkg.Solver(pkg.cavity_config(n))
    s.init((rho, z, z, z))
    s.step(3)
    assert s.status() & pkg.STATUS_RHO_RANGE


@pytest.mark.parametrize("case", ["cavity_f32", "cavity_f16", "channel_thermal", "couette_periodic_x"])
def test_xface_fix_matches_boundary_path_bitwise(pkg, case):
    """Lanes on x = 0 and x = nx-1 either keep the plain pull and redo their
    x-crossing links, or send their whole warp down the boundary-class path.
    Both give the same bits."""
    out = []
    for xp in (0, -1):
        if case.startswith("cavity"):
            cfg = pkg.cavity_config(37, tau=0.6, lid=0.05, ny=21, nz=13, storage=case[-3:], xface=xp)
        elif case == "channel_thermal":
            cfg = pkg.channel_config(40, 18, 14, 0.6, u_in=0.05, thermal=True, T_in=1.0, tau_g=0.7,
                                     gbeta=(0.0, 1e-4, 0.0), xface=xp)
        else:
            faces = {f: {"kind": pkg.FACE_PERIODIC} for f in (0, 1)}
            faces.update({f: {"kind": pkg.FACE_WALL} for f in (2, 4, 5)})
            faces[3] = {"kind": pkg.FACE_WALL, "u": (0.05, 0.0, 0.0)}
            cfg = pkg.make_config(24, 16, 12, 0.7, "f32", faces, xface=xp)
        s = pkg.Solver(cfg)
        s.init()
        s.step(1)
        s.step(70)
        assert s.status() == 0
        out.append(s.moments())
    for c in out[0]:
        assert np.array_equal(out[0][c], out[1][c]), c
