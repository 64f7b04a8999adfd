"""Batched cavities (lbmgpu_batch_*): every cavity of an uneven batch, advanced
by the shared persistent launches, equals the same cavity solved alone, and
matches the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_single_solves_and_oracle(pkg, orc):
    rng = np.random.default_rng(3)
    dims = rng.integers(8, 20, size=(6, 3))
    taus = rng.uniform(0.55, 0.9, size=6)
    steps = 120
    b = pkg.Batch(dims, taus, lid=0.05, storage="f32")
    b.init()
    b.step(steps)
    assert (b.status() == 0).all()
    for p in range(len(taus)):
        nx, ny, nz = (int(v) for v in dims[p])
        m = b.moments(p)
        s = pkg.Solver(pkg.cavity_config(nx, tau=float(taus[p]), lid=0.05, ny=ny, nz=nz))
        s.init()
        s.step(steps)
        ms = s.moments()
        lat = orc.cavity(nx, float(taus[p]), 0.05, ny=ny, nz=nz)
        lat.step_plain(steps)
        r = orc.moments(lat)
        for c in ("ux", "uy", "uz"):
            assert np.abs(m[c] - r[c]).max() / 0.05 < 1e-5, (p, c)
            assert np.abs(m[c] - ms[c]).max() / 0.05 < 1e-6, (p, c)


def test_batch_autotune_and_fp16(pkg, orc):
    rng = np.random.default_rng(5)
    dims = rng.integers(16, 40, size=(12, 3))
    taus = rng.uniform(0.52, 0.7, size=12)
    b = pkg.Batch(dims, taus, lid=0.05, storage="f16")
    threads, grid = b.autotune()
    assert threads in (128, 256, 512) and grid > 0
    b.init()
    b.step(200)
    p = 3
    nx, ny, nz = (int(v) for v in dims[p])
    m = b.moments(p)
    lat = orc.cavity(nx, float(taus[p]), 0.05, ny=ny, nz=nz)
    lat.step_plain(200)
    r = orc.moments(lat)
    assert np.abs(m["ux"] - r["ux"]).max() / 0.05 < 2e-3


def test_batch_flags_diverging_cavity(pkg):
    """A cavity that goes unstable is flagged in its own status word; the
    others are unaffected (failure reported, never trapped)."""
    dims = np.array([[12, 12, 12], [12, 12, 12]])
    taus = np.array([0.8, 0.5000001])
    b = pkg.Batch(dims, taus, lid=0.1, storage="f32")
    b.init()
    b.step(3000)
    st = b.status()
    assert st[0] == 0
    assert st[1] & pkg.STATUS_RHO_RANGE
