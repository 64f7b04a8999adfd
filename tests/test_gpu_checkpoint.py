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


@pytest.mark.parametrize("free", [False, True], ids=["fixed", "free_thermal"])
def test_sphere_restart_is_bitwise(pkg, orc, tmp_path, free):
    """IBM sphere, fixed or free in six degrees of freedom with the D3Q7
    population (force history, markers and the FP64 body restored).  The
    spreading sums in 64-bit fixed point, independent of the order of the
    atomics, so the continuation equals the uninterrupted run bit for bit."""
    nx, ny, nz, D, nm = 48, 32, 28, 8.0, 201
    center = (14.0, 16.0, 14.0)
    mk = orc.fibonacci_sphere(nm, D, center)
    xyz = np.stack([mk["x"], mk["y"], mk["z"]])

    def solver():
        kw = dict(thermal=True, tau_g=0.7, T_in=0.0, gbeta=(0.0, 1e-5, 0.0)) if free else {}
        s = pkg.Solver(pkg.channel_config(nx, ny, nz, 0.56, u_in=0.05, **kw))
        mkw = {}
        if free:
            vol = np.pi * D ** 3 / 6.0
            mkw = dict(free_body=True, density_ratio=1.5, volume=vol, inertia=0.4 * 1.5 * vol * (D / 2) ** 2,
                       gravity=(0.0, -1e-5, 0.0), free_dofs=63, virtual_mass=1.0, thermal=True, T_body=1.0)
        s.set_markers(xyz, mk["ds"], D / 2.0, center, m_max=3, **mkw)
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
    assert a.status() == 0 and b.status() == 0
    fa, fb = a.forces(), b.forces()
    assert fa.shape == fb.shape == (60, 8)
    assert np.array_equal(fa, fb)
    ma, mb = a.moments(), b.moments()
    for c in ma:
        assert np.array_equal(ma[c], mb[c]), c
    if free:
        assert np.array_equal(a.body(), b.body())
        assert np.array_equal(a.markers(), b.markers())


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


@pytest.mark.parametrize("case", ["cylinder", "transverse", "energy", "energy_neumann", "staircase"])
def test_d2q9_restart_is_bitwise(pkg, orc, tmp_path, case):
    """D2Q9 handles: the reference's default cylinder (fixed body, nearest-node
    density, added mass), its transverse oscillation (moving markers and box),
    the ENERGY Couette channel (g and the per-cell history) and the tandem
    staircase circles (interior solid cells); saved after 30 steps, restored
    onto a fresh handle of the same set-up, 30 more steps equal the
    uninterrupted run bit for bit."""
    import os

    from conftest import GOLDEN

    def make():
        if case in ("cylinder", "transverse"):
            from test_gpu_d2q9 import _cylinder_solver

            if case == "cylinder":
                g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
                return _cylinder_solver(pkg, orc, g, m_max=int(g["m_max"]))[0]
            g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_transverse_100.npz"))
            D = float(g["D"])
            return _cylinder_solver(pkg, orc, g, m_max=5, u_max=0.05, Re=100.0, marker_dy=2.0,
                                    vsolid=orc.REF_PI * D * D * 0.25 * 3, motion=pkg.MOTION_TRANSVERSE_OSC,
                                    motion_amp=2.0, motion_freq=0.005)[0]
        if case.startswith("energy"):
            from test_gpu_energy import _solver

            # a Neumann wall's cells keep last sweep's g: saved with the state
            top = orc.TYPE_Q if case == "energy_neumann" else None
            return _solver(pkg, orc, 30, 20.0, tau=0.8, nx=6, top=top)[0]
        from test_gpu_d2q9 import STAIRCASE, _staircase_gpu

        return _staircase_gpu(pkg, orc, [c for c in STAIRCASE if c[0] == "tandem"][0])[0]

    path = str(tmp_path / "d2.ckpt")
    a = make()
    a.step(30)
    a.save_state(path)
    a.step(30)
    b = make()
    b.load_state(path)
    b.step(30)
    assert a.status() == 0 and b.status() == 0
    ma, mb = a.moments(), b.moments()
    for c in ma:
        assert np.array_equal(ma[c], mb[c]), c
    if case in ("cylinder", "transverse"):
        assert np.array_equal(a.forces(), b.forces())
        assert np.array_equal(a.markers(), b.markers())
    if case.startswith("energy"):
        assert np.array_equal(a.download_f32(pkg.FIELD_QX), b.download_f32(pkg.FIELD_QX))


def test_d2q9_restart_rejects_other_files(pkg, orc, tmp_path):
    """A D3Q19 state file, or one of another D2Q9 lattice, is refused."""
    from test_gpu_energy import _solver

    p3 = str(tmp_path / "c3.ckpt")
    a = pkg.Solver(pkg.cavity_config(16, tau=0.7))
    a.init()
    a.step(2)
    a.save_state(p3)
    s, _ = _solver(pkg, orc, 30, 20.0, tau=0.8, nx=6)
    with pytest.raises(pkg.LbmError) as e:
        s.load_state(p3)
    assert e.value.status == 1
    p2 = str(tmp_path / "c2.ckpt")
    s.step(3)
    s.save_state(p2)
    t, _ = _solver(pkg, orc, 20, 20.0, tau=0.8, nx=6)
    with pytest.raises(pkg.LbmError) as e:
        t.load_state(p2)
    assert e.value.status == 1
