"""The C++ drop-in facade (csrc/facade/LBM.h): the reference's own time loops
(main.cpp:195-221) driving the GPU through the C ABI, against the oracle."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def drivers(pkg):
    import importlib.util

    p = os.path.join(os.path.dirname(pkg.__file__), "csrc", "facade", "build_facade.py")
    spec = importlib.util.spec_from_file_location("build_facade", p)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return dict(zip(m.DRIVERS, m.build()))


def test_dropin_cavity_loop(drivers, orc, tmp_path):
    n, steps = 16, 200
    out = str(tmp_path / "cav.bin")
    subprocess.check_call([drivers["dropin_cavity"], str(n), str(steps), out])
    g = orc.read_dropin_cavity(out, n)
    lat = orc.cavity(n, 0.8, 0.05)
    lat.step_plain(steps)
    r = orc.moments(lat)
    for c in ("ux", "uy", "uz"):
        assert np.abs(g[c] - r[c]).max() / 0.05 < 1e-5
    assert np.abs(g["rho"] - r["rho"]).max() < 1e-5


def test_dropin_sphere_ibm_loop(drivers, orc, tmp_path):
    nx, ny, nz, tau, D, nm, steps = 48, 28, 28, 0.56, 8.0, 201, 60
    out = str(tmp_path / "cd.csv")
    subprocess.check_call([drivers["dropin_sphere"], str(nx), str(ny), str(nz), str(tau), str(D), str(nm),
                           str(steps), out])
    cd = np.loadtxt(out, delimiter=",", skiprows=1)
    assert cd.shape == (steps, 3)
    center = (nx / 4.0, ny / 2.0, nz / 2.0)
    lat, mk, hist, _ = orc.sphere_case(nx, ny, nz, tau, D, center, nm, 5, 0.05, steps, outlet=orc.TYPE_OUT)
    q = 0.5 * 0.05 ** 2 * orc.REF_PI * D * D / 4
    ref_cd = hist[:, 0] / q
    assert np.abs(cd[:, 1] - ref_cd).max() / np.abs(ref_cd).max() < 1e-3


def test_dropin_staircase_sphere_loop(drivers, tmp_path):
    """The reference's Sphere_BB set-up and loop with MEA_CL / MEA_CD after
    every step, through the facade, against the reference's own run."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "sphere_bb48x24x24_D8_Re20_100.npz"))
    out = str(tmp_path / "mea.csv")
    subprocess.check_call([drivers["dropin_sphere_bb"], str(int(g["nx"])), str(int(g["ny"])), str(int(g["nz"])),
                           str(float(g["D"])), str(float(g["Re"])), str(float(g["u"])), str(int(g["steps"])), out])
    r = np.loadtxt(out, delimiter=",", skiprows=1)
    assert r.shape == (int(g["steps"]), 3)
    scale = np.abs(g["cd"]).max()
    assert np.abs(r[:, 2] - g["cd"]).max() / scale < 1e-4
    assert np.abs(r[:, 1] - g["cl"]).max() / scale < 1e-4


def test_dropin_more_details_loop(drivers, pkg, tmp_path):
    """The loop of a MORE_DETAILS build (Sup_MacroProp every Nt steps,
    main.cpp:389), through the facade compiled with -DMORE_DETAILS: the
    LATTICE fields pressure, sigma, avg_* and rms_* against the reference's
    own MORE_DETAILS run, and its OutputAVGVTK file."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "cavity8_details_200.npz"))
    n, steps = int(g["n"]), int(g["steps"])
    out = str(tmp_path / "det.bin")
    subprocess.check_call([drivers["dropin_details"], str(n), str(steps), out], cwd=str(tmp_path))
    a = np.fromfile(out, dtype=np.float64).reshape(36, n, n, n)
    inner = (Ellipsis, slice(1, -1), slice(1, -1), slice(1, -1))
    sym9 = [0, 1, 2, 1, 3, 4, 2, 4, 5]
    lid = float(g["lid"])
    assert np.abs(a[0] - g["p"][inner]).max() < 1e-7
    assert np.abs(a[1:10] - g["sigma"][sym9][inner]).max() < 1e-7
    assert np.abs(a[10:13] - g["avg_u"][inner]).max() < 2e-6 * lid
    assert np.abs(a[13] - g["avg_p"][inner]).max() < 1e-7
    assert np.abs(a[14:23] - g["avg_rs"][sym9][inner]).max() < 2e-6 * lid * lid
    assert np.abs(a[23:26] - g["rms_u"][inner]).max() < 2e-6 * lid
    assert np.abs(a[26] - g["rms_p"][inner]).max() < 1e-7
    assert np.abs(a[27:36] - g["rms_rs"][sym9][inner]).max() < 2e-6 * lid * lid
    v = pkg.read_vtr(str(tmp_path / "avgfield.vtr"))
    assert "Avg reynolds Stress" in v and v["CellType"].shape == ((n + 2) * (n + 2) * n,)


@pytest.mark.parametrize("case", ["fixed", "transverse"])
def test_dropin_cylinder2d_loop(drivers, tmp_path, case):
    """The reference's shipped default build (#define D2Q9, Cylinder_IBM,
    implicit forcing) and its transverse-oscillation variant, set up and run
    by the reference's own loop through the facade built with -DD2Q9: Cd / Cl
    after every step against the reference's runs."""
    from conftest import GOLDEN

    if case == "fixed":
        g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
        extra = []
    else:
        g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_transverse_100.npz"))
        extra = ["0", "transverse", "2.0", "0.005"]
    out = str(tmp_path / "cd.csv")
    subprocess.check_call([drivers["dropin_cylinder2d"], "80", "40", "10", "40", "5", str(int(g["steps"])), out] +
                          extra)
    r = np.loadtxt(out, delimiter=",", skiprows=1)
    assert r.shape == (int(g["steps"]), 3)
    scale = np.abs(g["cd"]).max()
    assert np.abs(r[:, 1] - g["cd"]).max() / scale < 2e-6
    assert np.abs(r[:, 2] - g["cl"]).max() / scale < 2e-6


def test_dropin_couette_neumann_loop(drivers, tmp_path):
    """The same build with the top wall's type_Energy TYPE_Q (a Neumann wall,
    j.n = 0): every fluid row against the reference's own single-thread run
    (1000 steps)."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "couette_neumann_ny30_re20_1000.npz"))
    ny = int(g["ny"])
    out = str(tmp_path / "couette_neumann.bin")
    subprocess.check_call([drivers["dropin_couette"], str(ny), str(float(g["Re"])), str(int(g["steps"])), out,
                           "neumann"], cwd=str(tmp_path))
    a = np.fromfile(out, dtype=np.float64).reshape(8, ny, 4)
    T = g["T"][1:-1]
    assert np.abs(a[4] - T).max() < 1e-3 * (T.max() - T.min())
    uw = np.abs(g["u"][0]).max()
    assert np.abs(a[1:4] - g["u"][:, 1:-1]).max() < 1e-5 * uw
    q = g["q"][:, 1:-1]
    assert np.abs(a[5:8] - q).max() < 1e-5 * np.abs(q).max()


def test_dropin_couette_energy_loop(drivers, tmp_path):
    """The reference's Couette_Flow build with its ENERGY model (-DD2Q9
    -DENERGY): main_setup_Couette's type_Energy / T set-up and the main loop
    through the facade; rho, u, T and q of every fluid row against the
    reference's own run (T within 1e-3 of the temperature spread: FP32)."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "couette_energy_ny30_re20_2000.npz"))
    ny = int(g["ny"])
    out = str(tmp_path / "couette.bin")
    subprocess.check_call([drivers["dropin_couette"], str(ny), str(float(g["Re"])), str(int(g["steps"])), out],
                          cwd=str(tmp_path))
    a = np.fromfile(out, dtype=np.float64).reshape(8, ny, 4)
    T = g["T"][1:-1]
    assert np.abs(a[4] - T).max() < 1e-3 * (T.max() - T.min())
    uw = np.abs(g["u"][0]).max()
    assert np.abs(a[0] - g["rho"][1:-1]).max() < 1e-5
    assert np.abs(a[1:4] - g["u"][:, 1:-1]).max() < 1e-5 * uw
    q = g["q"][:, 1:-1]
    assert np.abs(a[5:8] - q).max() < 1e-5 * np.abs(q).max()


@pytest.mark.parametrize("case", [("cylbasic", 100, 60, 20, 200.0, 0.1, 1), ("tandem", 160, 100, 10, 100.0, 0.05, 2),
                                  ("triangle", 100, 80, 10, 100.0, 0.05, 3)], ids=lambda c: c[0])
def test_dropin_staircase2d_loop(drivers, tmp_path, case):
    """The reference's staircase 2D cases with the momentum-exchange
    algorithm, set up by its own code pattern (Generate_Cylinder /
    Generate_Circle / Generate_Triangle and the face loops) and run by its
    loop through the facade built with -DD2Q9: MEA_CL / MEA_CD of every body
    in its box after every step against the reference's runs."""
    from conftest import GOLDEN

    kind, nx, ny, D, Re, u, nb = case
    g = np.load(os.path.join(GOLDEN, "staircase2d_%s_300.npz" % kind))
    steps = int(g["steps"])
    out = str(tmp_path / "mea.bin")
    subprocess.check_call([drivers["dropin_staircase2d"], kind, str(nx), str(ny), str(D), str(Re), str(u), "1.5",
                           str(nb), str(steps), out])
    a = np.fromfile(out).reshape(2, nb, steps)
    scale = np.abs(g["cd"]).max()
    assert np.abs(a[0] - g["cl"]).max() < 2e-5 * scale
    assert np.abs(a[1] - g["cd"]).max() < 2e-5 * scale


def test_dropin_poiseuille_energy_loop(drivers, tmp_path):
    """The reference's Poiseuille_Flow build with ENERGY (-DD2Q9 -DENERGY):
    main_setup_Poiseuille's set-up (F[0] = -dp/dx on the fluid cells, read
    as the body force) and loop through the facade, the walls moving at F/2
    from the third streaming (wall_force); rho, u, T against the reference's
    own run."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "poiseuille_ny30_re20_energy_1500.npz"))
    ny = int(g["ny"])
    out = str(tmp_path / "pois.bin")
    subprocess.check_call([drivers["dropin_poiseuille"], str(ny), str(float(g["Re"])), str(int(g["steps"])), out])
    a = np.fromfile(out, dtype=np.float64).reshape(8, ny, 4)
    um = np.abs(g["u"][0, 1:-1]).max()
    assert np.abs(a[1:3] - g["u"][:2, 1:-1]).max() < 3e-5 * um
    T = g["T"][1:-1]
    assert np.abs(a[4] - T).max() < 5e-3 * (T.max() - T.min())


def test_dropin_cylinder2d_outputs(drivers, pkg, tmp_path):
    """The default build's output calls through the facade (main.cpp:62-66,
    205-237): OutputVTK every Nt = 10 steps against the reference's own
    field file after 100 steps, OutputVTK_Marker's wall_t file against the
    reference's text, and OutputCSV's Cd / Cl files (time = (i + 1) u_max / D,
    six significant digits) against the reference's coefficients."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "cylinder80x40_vtk_100.npz"))
    c = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    steps = int(g["steps"])
    subprocess.check_call([drivers["dropin_cylinder2d"], "80", "40", "10", "40", "5", str(steps),
                           str(tmp_path / "cd.csv"), "0", "vtk", "10"], cwd=str(tmp_path))
    for n in range(steps // 10 + 1):
        assert (tmp_path / ("field%06d.vtr" % n)).exists(), n
        assert (tmp_path / ("wall_t %d.vtk" % n)).exists(), n
    v = pkg.read_vtr(str(tmp_path / ("field%06d.vtr" % (steps // 10))))
    assert v["header"] == str(g["header"])
    assert np.array_equal(v["CellType"], g["CellType"])
    assert np.abs(v["Density"] - g["Density"]).max() < 1e-5
    assert np.abs(v["Velocity"] - g["Velocity"]).max() * 0.1 < 1e-5  # u / u_max
    fscale = np.abs(g["Force density"]).max()
    assert np.abs(v["Force density"] - g["Force density"]).max() < 1e-5 * max(fscale, 1e-3) + 1e-7
    assert (tmp_path / str(g["marker_file_name"])).read_text() == str(g["marker_file"])
    for coef in ("cd", "cl"):
        r = np.loadtxt(str(tmp_path / ("C%s at Re = 40.000000.csv" % coef[1])), delimiter=",", skiprows=1)
        assert r.shape == (steps, 2)
        assert np.allclose(r[:, 0], (np.arange(steps) + 1) * 0.1 / 10.0, rtol=1e-5)
        scale = np.abs(c["cd"]).max()
        assert np.abs(r[:, 1] - c[coef]).max() / scale < 1e-5


def test_dropin_rayleigh_benard_loop(drivers, tmp_path):
    """The reference's Rayleigh_Benard build (-DENERGY on D3Q19):
    main_setup_RayleighBenard1 and the main loop with Find_Maximum_uy and
    Find_Nusselt_number every Nt steps, each time rewritten to the loop's CSV
    files (main.cpp:226, 308-321), through the facade,
    which hands the set-up to lbm_energy3d; every cell, ghosts included,
    against the reference's own run (FP32: T within 1e-5 of the spread, u
    within 1e-4 of its largest value), and the last recorded maximum |uy| and
    Nusselt number against the same formulas on the reference's fields."""
    from conftest import GOLDEN

    g = np.load(os.path.join(GOLDEN, "rayleigh32x16x5_400.npz"))
    nx, ny, nz, steps = int(g["nx"]), int(g["ny"]), int(g["nz"]), int(g["steps"])
    out = str(tmp_path / "rb.bin")
    r = subprocess.run([drivers["dropin_rayleigh"], str(nx), str(ny), str(nz), str(steps), out],
                       cwd=str(tmp_path), capture_output=True, text=True, check=True)
    info = json.loads(r.stdout.strip().splitlines()[-1])
    shape = (nz + 2, ny + 2, nx + 2)
    n = int(np.prod(shape))
    raw = np.fromfile(out, dtype=np.float64)
    a = raw[:8 * n].reshape((8,) + shape)
    rec = steps // 10
    uy_max, nus = raw[8 * n:8 * n + rec], raw[8 * n + rec:]
    assert uy_max.shape == (rec,) and nus.shape == (rec,)
    # the loop's CSV files, rewritten every Nt = 10 steps: time (i + 1) Nt dt
    for name, series in (("Maximum velocity in y direction at Ra = 1710.000000.csv", uy_max),
                         ("Nusselt number at Ra = 1710.000000.csv", nus)):
        r = np.loadtxt(str(tmp_path / name), delimiter=",", skiprows=1)
        assert (tmp_path / name).read_text().startswith("time,error\n")
        assert np.array_equal(r[:, 0], 10.0 * (np.arange(rec) + 1))
        assert np.allclose(r[:, 1], series, rtol=1e-5, atol=0)
    T = g["T"]
    assert np.abs(a[4] - T).max() < 1e-5 * (T.max() - T.min())
    us = np.abs(g["u"]).max()
    assert np.abs(a[1:4] - g["u"]).max() < 1e-4 * us
    assert np.abs(a[0] - g["rho"]).max() < 1e-6
    assert np.abs(a[5:8] - g["q"]).max() < 1e-4 * np.abs(g["q"]).max()
    # Find_Maximum_uy: every cell, ghosts included (lbm.cpp:3522-3536)
    assert abs(uy_max[-1] - np.abs(g["u"][1]).max()) < 1e-4 * np.abs(g["u"][1]).max()
    # Find_Nusselt_number (lbm.cpp:3538-3561) on the reference's fields
    cs2, Pr, Ra, gb = 1.0 / 3.0, 0.71, 1710.0, 1e-5
    nu = np.sqrt(gb * 1.0 * (nz + 1) ** 3 * Pr / Ra)
    alpha = nu / Pr
    fl = np.zeros(shape, bool)
    fl[1:-1, 1:-1, 1:-1] = True
    nu_ref = 1 + (g["u"][1][fl] * T[fl]).mean() / (alpha * 1.0 / (ny + 1))
    assert abs(nus[-1] - nu_ref) < 1e-4 * abs(nu_ref - 1.0), (nus[-1], nu_ref)
    # the ENERGY helpers on the mirror (fields from the dump, k, j, i order):
    # Determine_Wall_Temperature of cell (1, 1, 1), the mean T of its solid
    # neighbours (the walls as MacroProp leaves them), and Calc_geq along +y
    cxyz = [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (-1, -1, 0),
            (1, 0, 1), (-1, 0, -1), (0, 1, 1), (0, -1, -1), (1, -1, 0), (-1, 1, 0), (1, 0, -1), (-1, 0, 1),
            (0, 1, -1), (0, -1, 1)]
    solid = ~fl
    Ts = [a[4][1 + c[2], 1 + c[1], 1 + c[0]] for c in cxyz if solid[1 + c[2], 1 + c[1], 1 + c[0]]]
    assert abs(info["wall_T_1_1_1"] - np.mean(Ts)) < 1e-12
    rho, uy, Tc = a[0][1, 1, 1], a[2][1, 1, 1], a[4][1, 1, 1]
    uu = a[1][1, 1, 1] ** 2 + uy ** 2 + a[3][1, 1, 1] ** 2
    geq = rho / 18 * Tc * (1 + 3 * uy + 4.5 * uy ** 2 - 1.5 * uu + 4.5 * uy ** 3 - 4.5 * uy * uu)
    assert abs(info["geq_1_1_1_3"] - geq) < 1e-12 * abs(geq)
