"""GPU parity for the MORE_DETAILS mode (LBM.h:55): pressure and viscous
stress of MacroProp (lbm.cpp:681-705), the Sup_MacroProp running statistics
(lbm.cpp:865-939) and the MORE_DETAILS VTK files (OutputVTK, lbm.cpp:2290-2642;
OutputAVGVTK, lbm.cpp:2644-3031), against the reference's own MORE_DETAILS
run of the 8^3 cavity (tests/golden) and the FP64 oracle.

Tolerances (FP32 populations against the reference's FP64; measured errors
in brackets): pressure and stress within 1e-7 absolute [2.8e-8, 2.3e-8]
(|sigma_xx| ~ 0.125, |sigma_xy| up to 3e-3); velocity averages and rms
within 2e-6 U [1.8e-7 U]; pressure statistics within 1e-7 [2.2e-8];
Reynolds-stress statistics within 2e-6 U^2 [3.5e-7 U^2].  FP16 / BF16
storage: off-diagonal stress within 2e-3 / 2e-2 of max |sigma_xy|
[7.2e-4 and 3.1e-3]."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TOL_P = 1e-7
TOL_U = 2e-6


def _golden():
    return np.load(os.path.join(GOLDEN, "cavity8_details_200.npz"))


def _run_cavity(pkg, g, storage="f32", steps=None, graph_steps=0, solver=None, start=1):
    n, tau, lid, nt = int(g["n"]), float(g["tau"]), float(g["lid"]), int(g["nt"])
    steps = int(g["steps"]) if steps is None else steps
    s = solver
    if s is None:
        s = pkg.Solver(pkg.cavity_config(n, tau=tau, lid=lid, storage=storage, graph_steps=graph_steps))
        s.set_more_details(True)
        s.init()
    for step in range(start, steps + 1):
        s.step(1)
        if step % nt == 0:
            s.sup_macroprop(step, nt, 1.0)
    return s


def _inner(a):
    return a[..., 1:-1, 1:-1, 1:-1]


def test_details_and_statistics_vs_reference(pkg):
    g = _golden()
    lid = float(g["lid"])
    s = _run_cavity(pkg, g)
    assert s.status() == 0
    d = s.details()
    ep = np.abs(d["p"] - _inner(g["p"])).max()
    es = np.abs(d["sigma"] - _inner(g["sigma"])).max()
    st = s.stats()
    assert st["samples"] == 20 and st["told"] == 190.0
    err = {k: np.abs(st[k] - _inner(g[k])).max() for k in ("avg_u", "rms_u", "avg_p", "rms_p", "avg_rs", "rms_rs")}
    print("details errors: p %.3g sigma %.3g" % (ep, es), {k: "%.3g" % v for k, v in err.items()})
    assert ep < TOL_P and es < TOL_P, (ep, es)
    assert err["avg_u"] < TOL_U * lid and err["rms_u"] < TOL_U * lid
    assert err["avg_p"] < TOL_P and err["rms_p"] < TOL_P
    assert err["avg_rs"] < TOL_U * lid * lid and err["rms_rs"] < TOL_U * lid * lid


@pytest.mark.parametrize("storage,tol", [("f16", 2e-3), ("bf16", 2e-2)])
def test_details_half_storage(pkg, storage, tol):
    """FP16 / BF16 shifted storage: the stress off the diagonal within tol of
    the largest |sigma_xy| of the reference run."""
    g = _golden()
    s = _run_cavity(pkg, g, storage=storage)
    d = s.details()
    scale = np.abs(_inner(g["sigma"])[1]).max()
    e = np.abs(d["sigma"][[1, 2, 4]] - _inner(g["sigma"])[[1, 2, 4]]).max() / scale
    print(storage, "off-diagonal stress error / max |sigma_xy|: %.3g" % e)
    assert e < tol


def test_more_details_vtk_matches_reference_file(pkg, tmp_path):
    """OutputVTK in MORE_DETAILS mode against the reference's own file of the
    same run: the same header, and every array -- ghost cells included."""
    g = _golden()
    s = _run_cavity(pkg, g)
    path = str(tmp_path / "field000000.vtr")
    s.output_vtk_async(path, u_ref=0.1)  # the reference divides by its u_max = 0.1
    s.output_wait()
    v = pkg.read_vtr(path)
    assert v["header"] == str(g["vtk_header"])
    for k in ("CellType", "CoordinateX", "CoordinateY", "CoordinateZ", "Vorticity"):
        assert np.array_equal(v[k], g["vtk_" + k]), k
    assert np.abs(v["Density"] - g["vtk_Density"]).max() < 1e-6
    assert np.abs(v["Velocity"] - g["vtk_Velocity"]).max() * 0.1 < TOL_U * float(g["lid"])
    assert np.abs(v["Pressure"] - g["vtk_Pressure"]).max() < TOL_P
    assert np.abs(v["Viscous Stress"] - g["vtk_Viscous Stress"]).max() < TOL_P


def test_avg_vtk_layout_and_values(pkg, tmp_path):
    """OutputAVGVTK: the reference's array list and scaling, and the values of
    every cell (ghosts included) against the reference's statistics."""
    g = _golden()
    lid, u_ref = float(g["lid"]), 0.1
    s = _run_cavity(pkg, g)
    path = str(tmp_path / "avgfield.vtr")
    s.output_avg_vtk(path, u_ref=u_ref)
    v = pkg.read_vtr(path)
    names = ["Density", "Velocity", "Avg velocity", "Rms velocity", "Pressure", "Avg pressure", "Rms pressure",
             "Viscous Stress", "Vorticity", "Avg vorticity", "Rms vorticity", "Avg reynolds Stress",
             "Rms reynolds Stress", "CellType"]
    found = [n for n in v["header"].split('Name="')[1:]]
    assert [f.split('"')[0] for f in found[:len(names)]] == names
    n = int(g["n"])
    sh = (n, n + 2, n + 2)  # planes k = 1..Nz, every j and i

    def planes(a):  # ghost-inclusive golden -> file cells
        return a[..., 1:-1, :, :]

    def vec(a, comps):
        return np.moveaxis(planes(a), 0, -1).reshape(-1) if comps > 1 else planes(a).reshape(-1)

    sym9 = [0, 1, 2, 1, 3, 4, 2, 4, 5]
    assert np.abs(v["Avg velocity"] - vec(g["avg_u"], 3) / u_ref).max() * u_ref < TOL_U * lid
    assert np.abs(v["Rms velocity"] - vec(g["rms_u"], 3) / u_ref).max() * u_ref < TOL_U * lid
    assert np.abs(v["Avg pressure"] - vec(g["avg_p"], 1)).max() < TOL_P
    assert np.abs(v["Rms pressure"] - vec(g["rms_p"], 1)).max() < TOL_P
    for key, name in (("avg_rs", "Avg reynolds Stress"), ("rms_rs", "Rms reynolds Stress")):
        ref = vec(g[key][sym9], 9) / (u_ref * u_ref)
        assert np.abs(v[name] - ref).max() * u_ref * u_ref < TOL_U * lid * lid, name
    for name in ("Vorticity", "Avg vorticity", "Rms vorticity"):
        assert not v[name].any()
    assert v["Density"].shape == (np.prod(sh),)


def test_stress_staircase_sphere_vs_oracle(pkg, orc):
    """The solid-cell path (bounce-back pull, frozen solid cells) of the
    details pass against the oracle's restatement."""
    nx, ny, nz, D, u, tau, steps = 48, 24, 24, 8.0, 0.05, 0.56, 60
    lat, _ = orc.sphere_bb(nx, ny, nz, tau, D, u)
    cfg = pkg.config_from_types(nx, ny, nz, tau, lat.types.copy(), lat.rho.copy(), lat.ux.copy(), lat.uy.copy(),
                                lat.uz.copy())
    s = pkg.Solver(cfg)
    s.set_solids(lat.interior(lat.types) == orc.TYPE_S)
    s.set_more_details(True)
    s.init([lat.interior(getattr(lat, c)) for c in ("rho", "ux", "uy", "uz")])
    s.step(steps)
    lat.step_plain(steps)
    ref = orc.details(lat)
    d = s.details()
    ep = np.abs(d["p"] - lat.interior(ref["p"])).max()
    es = np.abs(d["sigma"] - ref["sigma"][:, 1:-1, 1:-1, 1:-1]).max()
    print("sphere details errors: p %.3g sigma %.3g" % (ep, es))
    assert ep < TOL_P and es < 2 * TOL_P


def test_statistics_survive_checkpoint(pkg, tmp_path):
    g = _golden()
    whole = _run_cavity(pkg, g, steps=120).stats()
    a = _run_cavity(pkg, g, steps=60)
    path = str(tmp_path / "det.ckpt")
    a.save_state(path)
    b = pkg.Solver(pkg.cavity_config(int(g["n"]), tau=float(g["tau"]), lid=float(g["lid"])))
    b.set_more_details(True)
    b.load_state(path)
    _run_cavity(pkg, g, steps=120, solver=b, start=61)
    st = b.stats()
    for k in ("avg_u", "rms_u", "avg_p", "rms_p", "avg_rs", "rms_rs", "samples", "told"):
        assert np.array_equal(st[k], whole[k]), k
    c = pkg.Solver(pkg.cavity_config(int(g["n"]), tau=float(g["tau"]), lid=float(g["lid"])))
    with pytest.raises(pkg.LbmError):
        c.load_state(path)  # saved in MORE_DETAILS mode, restored without it


def test_more_details_calls_need_the_mode(pkg):
    s = pkg.Solver(pkg.cavity_config(8))
    s.init()
    for call in (s.details, s.stats, lambda: s.sup_macroprop(10)):
        with pytest.raises(pkg.LbmError) as e:
            call()
        assert e.value.status == 6
    s.set_more_details(True)
    s.step(10)
    s.sup_macroprop(10)
    assert s.stats()["samples"] == 1
    s.set_more_details(False)
    with pytest.raises(pkg.LbmError):
        s.details()


def _triangle(pkg, orc):
    """The reference's Cylinder_Tandem_Triangle in MORE_DETAILS mode (D2Q9,
    60 x 40, two triangles), 200 steps with Sup_MacroProp every 10."""
    from test_gpu_d2q9 import _staircase_gpu

    g = np.load(os.path.join(GOLDEN, "triangle60x40_details_200.npz"))
    case = ("triangle", int(g["nx"]), int(g["ny"]), int(g["D"]), float(g["Re"]), float(g["u_in"]), int(g["nb"]))
    s = _staircase_gpu(pkg, orc, case)[0]
    s.set_more_details(True)
    nt = int(g["nt"])
    for step in range(1, int(g["steps"]) + 1):
        s.step(1)
        if step % nt == 0:
            s.sup_macroprop(step, nt, 1.0)
    assert s.status() == 0
    return s, g


def test_d2q9_details_vs_reference(pkg, orc):
    """D2Q9 handles: the pressure, the viscous stress and the Sup_MacroProp
    statistics of every interior cell against the reference's own
    MORE_DETAILS run of its tandem-triangle case (staircase solids, inlet and
    outlet faces, tau = 0.515).  The Reynolds-stress statistics are products
    of velocities: their FP32 error is about 2 U times that of u, so they are
    held to 2 U TOL_U U [measured 2.5e-6 U^2]."""
    s, g = _triangle(pkg, orc)
    u = float(g["u_in"])

    def inner(a):
        return a[..., 1:-1, 1:-1]

    d = s.details()
    ep = np.abs(d["p"][0] - inner(g["p"])).max()
    es = np.abs(d["sigma"][:, 0] - inner(g["sigma"])).max()
    st = s.stats()
    assert st["samples"] == 20 and st["told"] == 190.0
    err = {k: np.abs((st[k][:, 0] if st[k].ndim == 4 else st[k][0]) - inner(g[k])).max()
           for k in ("avg_u", "rms_u", "avg_p", "rms_p", "avg_rs", "rms_rs")}
    print("D2Q9 details errors: p %.3g sigma %.3g" % (ep, es), {k: "%.3g" % v for k, v in err.items()})
    assert ep < TOL_P and es < TOL_P, (ep, es)
    assert err["avg_u"] < TOL_U * u and err["rms_u"] < TOL_U * u
    assert err["avg_p"] < TOL_P and err["rms_p"] < TOL_P
    assert err["avg_rs"] < 2 * TOL_U * u * u and err["rms_rs"] < 2 * TOL_U * u * u


def test_d2q9_details_vtk_files_match_reference(pkg, orc, tmp_path):
    """OutputVTK and OutputAVGVTK of the D2Q9 MORE_DETAILS run against the
    reference's own files of the same run: the same headers, CellType and
    coordinates exactly, every other array within FP32 tolerance (ghost cells
    included): the velocities within 1e-5 U as the D2Q9 staircase fields
    [5.6e-6 U], the rest as test_d2q9_details_vs_reference."""
    s, g = _triangle(pkg, orc)
    u = float(g["u_in"])
    types = g["types"]
    path = str(tmp_path / "field000000.vtr")
    s.output_vtk_async(path, u_ref=u, types=types)
    s.output_wait()
    v = pkg.read_vtr(path)
    assert v["header"] == str(g["vtk_header"])
    for k in ("CellType", "CoordinateX", "CoordinateY", "CoordinateZ", "Vorticity"):
        assert np.array_equal(v[k], g["vtk_" + k]), k
    assert np.abs(v["Density"] - g["vtk_Density"]).max() < 1e-6
    assert np.abs(v["Velocity"] - g["vtk_Velocity"]).max() < 1e-5  # u / u_in
    assert np.abs(v["Pressure"] - g["vtk_Pressure"]).max() < TOL_P
    assert np.abs(v["Viscous Stress"] - g["vtk_Viscous Stress"]).max() < TOL_P
    apath = str(tmp_path / "avgfield.vtr")
    s.output_avg_vtk(apath, u_ref=u, types=types)
    w = pkg.read_vtr(apath)
    assert w["header"] == str(g["avgvtk_header"])
    for k in ("CellType", "CoordinateX", "CoordinateY", "CoordinateZ", "Vorticity", "Avg vorticity", "Rms vorticity"):
        assert np.array_equal(w[k], g["avgvtk_" + k]), k
    # velocities in the file are u / u_in, Reynolds stresses u u / u_in^2
    tol = {"Density": 1e-6, "Pressure": TOL_P, "Avg pressure": TOL_P, "Rms pressure": TOL_P,
           "Viscous Stress": TOL_P, "Velocity": 1e-5, "Avg velocity": 1e-5, "Rms velocity": 1e-5,
           "Avg reynolds Stress": 2e-5, "Rms reynolds Stress": 2e-5}
    for k, t in tol.items():
        e = np.abs(w[k] - g["avgvtk_" + k]).max()
        assert e < t, (k, e)
