"""Checkpoint and restart: a run saved at step n and restored onto a fresh
handle continues exactly as the uninterrupted run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["f32", "f16"])
def test_cavity_restart_is_bitwise(pkg, tmp_path, storage):
    path = str(tmp_path / "cav.ckpt")
    a = pkg.Solver(pkg.cavity_config(20, tau=0.7, lid=0.05, ny=16, nz=12, storage=storage, graph_steps=10))
    a.init()
    a.step(35)
    a.save_state(path)
    a.step(40)
    b = pkg.Solver(pkg.cavity_config(20, tau=0.7, lid=0.05, ny=16, nz=12, storage=storage, graph_steps=10))
    b.load_state(path)
    assert b.steps_done() == 35
    b.step(40)
    ma, mb = a.moments(), b.moments()
    for c in ma:
        assert np.array_equal(ma[c], mb[c]), c


def test_sphere_restart_continues(pkg, orc, tmp_path):
    """IBM sphere (force history and markers restored); the spreading sums in
    float atomics, so the continuation agrees to rounding."""
    nx, ny, nz, D, nm = 48, 32, 28, 8.0, 201
    center = (14.0, 16.0, 14.0)
    mk = orc.fibonacci_sphere(nm, D, center)
    xyz = np.stack([mk["x"], mk["y"], mk["z"]])

    def solver():
        s = pkg.Solver(pkg.channel_config(nx, ny, nz, 0.56, u_in=0.05))
        s.set_markers(xyz, mk["ds"], D / 2.0, center, m_max=3)
        return s

    path = str(tmp_path / "sph.ckpt")
    a = solver()
    a.init()
    a.step(30)
    a.save_state(path)
    a.step(30)
    b = solver()
    b.load_state(path)
    b.step(30)
    fa, fb = a.forces(), b.forces()
    assert fa.shape == fb.shape == (60, 8)
    assert np.array_equal(fa[:30], fb[:30])
    assert np.abs(fa[30:, :3] - fb[30:, :3]).max() / np.abs(fa[:, 0]).max() < 1e-4
    assert np.abs(a.moments()["ux"] - b.moments()["ux"]).max() / 0.05 < 1e-5


def test_restart_rejects_other_configuration(pkg, tmp_path):
    path = str(tmp_path / "c.ckpt")
    a = pkg.Solver(pkg.cavity_config(16, tau=0.7))
    a.init()
    a.step(3)
    a.save_state(path)
    b = pkg.Solver(pkg.cavity_config(16, tau=0.7, storage="f16"))
    with pytest.raises(pkg.LbmError) as e:
        b.load_state(path)
    assert e.value.status == 1
