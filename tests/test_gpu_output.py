"""Output in the reference's file formats: the asynchronous RectilinearGrid
writer against the reference's own OutputVTK file (lbm.cpp:2290-2642) of the
same cavity run, the snapshot semantics of the asynchronous path, and the
marker POLYDATA of OutputVTK_Marker (lbm.cpp:3033-3077)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_vtk_matches_reference_outputvtk(pkg, tmp_path):
    g = np.load(os.path.join(GOLDEN, "cavity12_vtk_200.npz"))
    s = pkg.Solver(pkg.cavity_config(12, tau=0.8, lid=0.05))
    s.init()
    s.step(200)
    path = str(tmp_path / "field000000.vtr")
    s.output_vtk_async(path, u_ref=0.1)  # the reference divides by its u_max = 0.1
    s.output_wait()
    v = pkg.read_vtr(path)
    assert v["header"] == str(g["header"])
    for k in ("CellType", "CoordinateX", "CoordinateY", "CoordinateZ"):
        assert np.array_equal(v[k], g[k]), k
    assert np.abs(v["Density"] - g["Density"]).max() < 1e-6
    # velocity / 0.1, FP32 against FP64: 1e-5 of the lid velocity
    assert np.abs(v["Velocity"] - g["Velocity"]).max() * 0.1 / 0.05 < 1e-5


def test_vtk_is_a_snapshot_of_the_call(pkg, tmp_path):
    """The file holds the state at the call even though the solver steps on
    before the writer finishes."""
    s = pkg.Solver(pkg.channel_config(40, 18, 14, 0.6, u_in=0.05, graph_steps=10))
    s.init()
    s.step(30)
    m = s.moments()
    path = str(tmp_path / "snap.vtr")
    s.output_vtk_async(path)
    s.step(50)
    s.output_wait()
    v = pkg.read_vtr(path)
    rho = v["Density"].reshape(14, 20, 42)[:, 1:-1, 1:-1]
    ux = v["Velocity"].reshape(14, 20, 42, 3)[:, 1:-1, 1:-1, 0]
    assert np.array_equal(rho, m["rho"].astype(np.float32))
    assert np.array_equal(ux, m["ux"].astype(np.float32))
    assert not np.array_equal(s.moments()["ux"], m["ux"])


def test_vtk_thermal_ibm_arrays_and_markers(pkg, orc, tmp_path):
    nx, ny, nz, D, nm = 48, 32, 28, 8.0, 201
    center = (14.0, 16.0, 14.0)
    s = pkg.Solver(pkg.channel_config(nx, ny, nz, 0.56, u_in=0.02, thermal=True, T_in=0.0, tau_g=0.6))
    s.init()
    mk = orc.fibonacci_sphere(nm, D, center)
    xyz = np.stack([mk["x"], mk["y"], mk["z"]])
    s.set_markers(xyz, mk["ds"], D / 2.0, center, m_max=3, thermal=True, T_body=1.0)
    s.step(20)
    path = str(tmp_path / "t.vtr")
    s.output_vtk_async(path, u_ref=0.02)
    s.output_wait()
    v = pkg.read_vtr(path)
    for k in ("Density", "Velocity", "Force density", "Temperature", "Heat flux", "CellType"):
        assert k in v and np.isfinite(v[k]).all(), k
    T = v["Temperature"].reshape(nz, ny + 2, nx + 2)[:, 1:-1, 1:-1]
    assert np.allclose(T, s.download(pkg.FIELD_T).astype(np.float32), atol=1e-6)
    fmag = np.abs(v["Force density"]).reshape(nz, ny + 2, nx + 2, 3).max()
    assert fmag > 0.0
    mpath = str(tmp_path / "wall.vtk")
    s.output_markers_vtk(mpath)
    lines = open(mpath).read().split("\n")
    assert lines[:5] == ["# vtk DataFile Version 3.0", "wall_state", "ASCII", "DATASET POLYDATA",
                         "POINTS %d float" % nm]
    pts = np.array([[float(t) for t in lines[5 + m].split()] for m in range(nm)])
    assert np.abs(pts - xyz.T).max() < 1e-4
    assert lines[5 + nm] == "LINES %d %d" % (nm, 3 * nm)


def test_vtk_d2q9_cylinder_matches_reference_outputvtk(pkg, orc, tmp_path):
    """The reference's default build (#define D2Q9, Cylinder_IBM): OutputVTK of
    the state after 100 steps against the reference's own file of the same
    run -- header byte for byte, CellType and coordinates exactly, Density,
    Velocity / u_max and the IBM Force density within FP32 tolerance -- and
    OutputVTK_Marker against the reference's marker file, text for text."""
    from test_gpu_d2q9 import _cylinder_gpu

    g = np.load(os.path.join(GOLDEN, "cylinder80x40_vtk_100.npz"))
    c = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    s, cl, cd = _cylinder_gpu(pkg, orc, c, int(g["steps"]), m_max=int(c["m_max"]))
    types = g["CellType"].reshape(42, 82).astype(np.uint8)
    path = str(tmp_path / "field000000.vtr")
    s.output_vtk_async(path, u_ref=0.1, types=types)  # the reference divides by its u_max = 0.1
    s.output_wait()
    v = pkg.read_vtr(path)
    assert v["header"] == str(g["header"])
    for k in ("CellType", "CoordinateX", "CoordinateY", "CoordinateZ"):
        assert np.array_equal(v[k], g[k]), k
    def worst(a, b):
        d = np.abs(a - b).reshape(42, 82, -1).max(axis=2)
        return d.max(), np.unravel_index(np.argmax(d), d.shape)

    assert worst(v["Density"], g["Density"])[0] < 1e-5, worst(v["Density"], g["Density"])
    # Velocity is u / u_max: 1e-5 in lattice units
    assert worst(v["Velocity"], g["Velocity"])[0] * 0.1 < 1e-5, worst(v["Velocity"], g["Velocity"])
    fscale = np.abs(g["Force density"]).max()
    assert fscale > 0
    assert np.abs(v["Force density"] - g["Force density"]).max() < 1e-5 * max(fscale, 1e-3) + 1e-7
    mpath = str(tmp_path / str(g["marker_file_name"]))
    s.output_markers_vtk(mpath)
    assert open(mpath).read() == str(g["marker_file"])
