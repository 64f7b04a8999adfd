"""The FP64 oracle against golden vectors produced by the reference itself.

The fixtures in tests/golden/ come from the reference's own lbm.cpp, built
unmodified by oracle/build_ref.sh and run by tests/golden/gen_golden.py.
These pin the restatement in oracle/lbm_oracle.c: the D3Q19 cavity path
(Init, Collision, Streaming with moving-wall bounce-back, MacroProp) and the
D2Q9 implicit IBM path (IBLBM with the reference's sign and rho_near
conventions, added mass, Cl/Cd).
"""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_cavity12_matches_reference(orc):
    g = np.load(os.path.join(GOLDEN, "cavity12_tau0.8_lid0.05_200.npz"))
    lat = orc.cavity(int(g["n"]), float(g["tau"]), float(g["lid"]))
    assert lat.step_plain(int(g["steps"])) == 0
    lid = float(g["lid"])
    assert np.abs(lat.interior(lat.rho) - g["rho"]).max() < 1e-12
    for c in ("ux", "uy", "uz"):
        assert np.abs(lat.interior(getattr(lat, c)) - g[c]).max() / lid < 1e-12


def _cylinder_literal(orc, g, steps):
    nx, ny, D, nodes, mm = int(g["nx"]), int(g["ny"]), float(g["D"]), int(g["nodes"]), int(g["m_max"])
    u_max = 0.1
    nu = u_max * D / 40.0
    tau = 0.5 + nu / (1.0 / 3.0)
    lat = orc.Lattice(9, nx, ny, 1, tau)
    t = lat.types
    # main_setup_Cylinder_IBM (lbm.cpp:1828-1854)
    t[:] = orc.TYPE_F
    t[:, :, 0] = orc.TYPE_IN
    t[:, :, -1] = orc.TYPE_OUT
    t[:, 0, :] = orc.TYPE_OUT
    t[:, -1, :] = orc.TYPE_OUT
    lat.ux[:] = u_max
    lat.init()
    cx, cy = nx / 5.0, ny / 2.0
    mk = orc.cylinder_markers_literal(nodes, D, cx, cy)
    lo = [math.floor(cx - D), math.floor(cy - D), 1]
    hi = [math.ceil(cx + D), math.ceil(cy + D), 1]
    op = orc.ibm_opts(lo, hi, mm, lit_sign=1, rho_mode=1)
    op.use_avg_density = 1
    op.vsolid = orc.REF_PI * D * D * 0.25
    cl, cd = [], []
    for _ in range(steps):
        out = lat.step_ibm(mk, op, [cx, cy, 1.0])
        cl.append(out[1] / (0.5 * u_max ** 2 * D))
        cd.append(out[0] / (0.5 * u_max ** 2 * D))
    return lat, mk, np.array(cl), np.array(cd)


def test_cylinder_ibm_matches_reference(orc):
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    lat, mk, cl, cd = _cylinder_literal(orc, g, int(g["steps"]))
    assert np.abs(mk["x"] - g["markers"][:, 0]).max() == 0.0
    assert np.abs(mk["nx"] - g["markers"][:, 3]).max() == 0.0
    assert np.abs(mk["ds"] - g["markers"][:, 6]).max() == 0.0
    for name, arr in (("rho", lat.rho), ("ux", lat.ux), ("uy", lat.uy), ("Fx", lat.Fx), ("Fy", lat.Fy)):
        assert np.abs(arr[1] - g[name]).max() < 1e-12, name
    assert np.abs(cd - g["cd"]).max() < 1e-10
    assert np.abs(cl - g["cl"]).max() < 1e-10


def test_kernel_is_peskin_4pt(orc):
    L = orc.lib()
    # partition of unity and first moment of the 4-point delta
    for r0 in (0.0, 0.1, 0.37, 0.5, 0.93):
        w = [L.orc_kernel(r0 - k) for k in range(-2, 3)]
        assert abs(sum(w) - 1.0) < 1e-14
        assert abs(sum(wi * (r0 - k) for wi, k in zip(w, range(-2, 3)))) < 1e-14
    assert L.orc_kernel(2.0) == 0.0 and L.orc_kernel(-2.5) == 0.0


def test_reference_literal_build_agrees_live(orc, tmp_path):
    """When the reference tree is present, rebuild and rerun it for a fresh case."""
    exe = os.path.join(orc.HERE, "_ref", "ref_cavity_12_0.8")
    if not os.path.exists(exe):
        pytest.skip("reference-literal oracle not built (no reference tree on this machine)")
    import subprocess

    out = str(tmp_path / "c.bin")
    subprocess.check_call([exe, "37", out, "0.03"], stdout=subprocess.DEVNULL)
    r = orc.read_ref_dump(out, 14, 14, 14, 4)["fields"]
    lat = orc.cavity(12, 0.8, 0.03)
    lat.step_plain(37)
    for w, a in enumerate((lat.rho, lat.ux, lat.uy, lat.uz)):
        assert np.abs(lat.interior(a) - r[w][1:-1, 1:-1, 1:-1]).max() < 1e-13


def test_staircase_sphere_mea_matches_reference(orc):
    """The reference's Sphere_BB case (staircase sphere, bounce-back on
    interior solid cells, TYPE_IN / TYPE_OUT ghosts) and its momentum-exchange
    Cl / Cd (MEA_CL / MEA_CD, lbm.cpp:3085-3163) after every step."""
    g = np.load(os.path.join(GOLDEN, "sphere_bb48x24x24_D8_Re20_100.npz"))
    nx, ny, nz, D, Re, u = int(g["nx"]), int(g["ny"]), int(g["nz"]), float(g["D"]), float(g["Re"]), float(g["u"])
    tau = 0.5 + (u * D / Re) / (1.0 / 3.0)
    lat, box = orc.sphere_bb(nx, ny, nz, tau, D, u)
    area = 0.5 * u * u * D * D * 3.14159265 / 4.0
    cl, cd = [], []
    for _ in range(int(g["steps"])):
        lat.collide()
        lat.stream()
        lat.macro()
        m = lat.mea(box)
        cl.append(m[1] / area)
        cd.append(-m[0] / area)
    assert np.abs(np.array(cd) - g["cd"]).max() < 1e-12 * np.abs(g["cd"]).max()
    assert np.abs(np.array(cl) - g["cl"]).max() < 1e-12 * np.abs(g["cd"]).max()
    f = np.stack([lat.interior(getattr(lat, c)) for c in ("rho", "ux", "uy", "uz")])
    assert np.abs(f[:, 12] - g["zmid"]).max() < 1e-12
    assert np.abs(f[:, :, 12] - g["ymid"]).max() < 1e-12
    assert np.allclose(f.reshape(4, -1).sum(axis=1), g["sums"], rtol=1e-12, atol=1e-12)


def test_more_details_match_reference(orc):
    """MORE_DETAILS mode of the reference (LBM.h:55) on the 8^3 cavity: the
    pressure and viscous stress of MacroProp (lbm.cpp:681-705) and the
    Sup_MacroProp running averages / rms values (lbm.cpp:865-939, called every
    Nt = 10 steps) at every cell, ghosts included.  The restatement sums in
    the reference's order: bit-exact."""
    g = np.load(os.path.join(GOLDEN, "cavity8_details_200.npz"))
    lat, det, st = orc.cavity_details_run(int(g["n"]), float(g["tau"]), float(g["lid"]), int(g["steps"]),
                                          int(g["nt"]))
    assert np.array_equal(lat.rho, g["rho"])
    assert np.array_equal(np.stack([lat.ux, lat.uy, lat.uz]), g["u"])
    assert np.array_equal(det["p"], g["p"])
    assert np.array_equal(det["sigma"], g["sigma"])
    for k in ("avg_u", "avg_p", "avg_rs", "rms_u", "rms_p", "rms_rs"):
        assert np.array_equal(getattr(st, k), g[k]), k
    # the reference's pressure-rms weighting (the current pressure squared
    # where the other rms values square their previous rms): on a ghost cell
    # at rest p = 1/3 and rms_p = p sqrt(told / (told + 1)), told = 190
    assert abs(g["rms_p"][0, 0, 0] - np.sqrt(190.0 / 191.0) / 3.0) < 1e-15


def test_triangle_details_matches_reference(orc):
    """The reference's Cylinder_Tandem_Triangle in MORE_DETAILS mode (D2Q9,
    triangled variant of oracle/build_ref.sh): after 200 steps with
    Sup_MacroProp every 10, rho, u, the pressure, the viscous stress and the
    running statistics of the k = 1 layer, within 1e-13 as the other staircase
    fixtures (measured 8e-16)."""
    g = np.load(os.path.join(GOLDEN, "triangle60x40_details_200.npz"))
    lat, det, st = orc.staircase2d_details_run("triangle", int(g["nx"]), int(g["ny"]), float(g["D"]),
                                               float(g["Re"]), float(g["u_in"]), int(g["steps"]), float(g["lpd"]),
                                               int(g["nb"]), int(g["nt"]))
    assert np.abs(lat.rho[1] - g["rho"]).max() < 1e-13
    assert np.abs(np.stack([lat.ux[1], lat.uy[1], lat.uz[1]]) - g["u"]).max() < 1e-13
    assert np.abs(det["p"][1] - g["p"]).max() < 1e-13
    assert np.abs(det["sigma"][:, 1] - g["sigma"]).max() < 1e-13
    for k in ("avg_u", "avg_p", "avg_rs", "rms_u", "rms_p", "rms_rs"):
        a = getattr(st, k)
        assert np.abs((a[:, 1] if a.ndim == 4 else a[1]) - g[k]).max() < 1e-13, k


def moving_case_kwargs(orc, case, D=10.0):
    """Cylinder2D options of the moving-body cases in fluid at rest."""
    if case == "inline":
        u, f = 5.0 * D * 1e-3, 1e-3
        return dict(m_max=5, u_max=u, Re=100.0, motion=orc.inline_motion(u, f), vsolid=orc.REF_PI * D * D * 0.25 * 3,
                    at_rest=True, center=(40.0, 20.0), area=D + 1.0)
    return dict(m_max=5, u_max=0.1, Re=40.0, motion=orc.towed_motion(0.1), at_rest=True, center=(80.0, 20.0))


@pytest.mark.parametrize("case", ["explicit", "transverse", "inline", "towed"])
def test_cylinder2d_variants_match_reference(orc, case):
    """The explicit direct-forcing scheme (lbm.cpp:1171-1258), the
    transversely oscillating cylinder (moving markers and box, added mass,
    markers generated at center_y + amplitude, lbm.cpp:1966), the inline
    oscillation (Cd over D + dx) and the towed cylinder, the last two in fluid
    at rest (TYPE_OUT on every face), against the reference's own runs."""
    win = (slice(8, 33), slice(4, 29))
    if case == "explicit":
        g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_explicit_100.npz"))
        kw = dict(m_max=1, scheme=1)
    elif case in ("inline", "towed"):
        g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_inline_100.npz" if case == "inline"
                                 else "cylinder120x40_D10_n40_m5_towed_100.npz"))
        kw = moving_case_kwargs(orc, case)
        nx = int(g["nx"])
        win = (slice(6, 36), slice(nx // 2 - 20, nx // 2 + 30))
    else:
        g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_transverse_100.npz"))
        D = float(g["D"])
        kw = dict(m_max=5, u_max=0.05, Re=100.0, motion=orc.transverse_motion(2.0, 0.005),
                  vsolid=orc.REF_PI * D * D * 0.25 * 3, marker_dy=2.0)
    lat, mk, cl, cd = orc.cylinder2d_literal(int(g["nx"]), int(g["ny"]), float(g["D"]), int(g["nodes"]),
                                             steps=int(g["steps"]), **kw)
    scale = np.abs(g["cd"]).max()
    assert np.abs(cd - g["cd"]).max() < 1e-12 * scale
    assert np.abs(cl - g["cl"]).max() < 1e-12 * scale
    assert np.abs(mk["y"] - g["markers"][:, 1]).max() == 0.0
    assert np.abs(mk["x"] - g["markers"][:, 0]).max() == 0.0
    f = np.stack([lat.rho[1], lat.ux[1], lat.uy[1], lat.Fx[1], lat.Fy[1]])
    assert np.abs(f[(slice(None),) + win] - g["window"]).max() < 1e-12
    assert np.allclose(f.reshape(5, -1).sum(axis=1), g["sums"], rtol=1e-12, atol=1e-12)


def test_energy_neumann_wall_matches_reference(orc):
    """The ENERGY Couette with its top wall a Neumann wall (type_Energy
    TYPE_Q, j.n = 0; Determine_Twall_Neumann, lbm.cpp:983-1028): the wall
    temperature from the cell's g in the middle of the push -- this sweep's
    values for the links whose source comes earlier in the (i, j, k) loop,
    last sweep's for the others --, the unknown g as the second-order
    equilibrium of T_w (lbm.cpp:281-288), T_w written into the wall cell.
    Against the reference run on one thread (its OpenMP split over i changes
    the result), bit for bit after 1000 steps, ghosts included."""
    g = np.load(os.path.join(GOLDEN, "couette_neumann_ny30_re20_1000.npz"))
    lat, c = orc.couette_energy(int(g["ny"]), float(g["Re"]), top=orc.TYPE_Q)
    assert lat.step_plain(int(g["steps"])) == 0
    assert np.array_equal(lat.rho[1], g["rho"])
    assert np.array_equal(np.stack([lat.ux[1], lat.uy[1], lat.uz[1]]), g["u"])
    assert np.array_equal(lat.T[1], g["T"])
    assert np.array_equal(lat.hq[:, 1], g["q"])
    # no heat crosses the top wall: the profile flattens towards it (about a
    # twentieth of the gradient at the Dirichlet bottom wall)
    T = g["T"][:, 1]
    assert abs(T[-2] - T[-3]) < 0.1 * abs(T[2] - T[1])


def test_energy_rayleigh_benard_matches_reference(orc):
    """The reference's Rayleigh_Benard case (main_setup_RayleighBenard1,
    lbm.cpp:1585-1643; LBM.h:222-242), D3Q19 with ENERGY: Dirichlet y walls,
    Neumann x and z walls whose T the push writes into the wall cells, read
    by the Dirichlet walls' Determine_Wall_Temperature of cells visited later
    (edges mix both kinds), and F_y = g beta (T - T*) refreshed by MacroProp
    on every cell, so that the walls report u = F / 2 and bounce back as
    moving walls from the third streaming on.  Against the reference run on
    one thread: bit for bit after 400 steps on a 32 x 16 x 5 box, ghosts
    included."""
    g = np.load(os.path.join(GOLDEN, "rayleigh32x16x5_400.npz"))
    lat, c = orc.rayleigh_benard(int(g["nx"]), int(g["ny"]), int(g["nz"]))
    assert lat.step_plain(int(g["steps"])) == 0
    assert np.array_equal(lat.rho, g["rho"])
    assert np.array_equal(np.stack([lat.ux, lat.uy, lat.uz]), g["u"])
    assert np.array_equal(np.stack([lat.Fx, lat.Fy, lat.Fz]), g["F"])
    assert np.array_equal(lat.T, g["T"])
    assert np.array_equal(lat.hq, g["q"])
    # the walls move at F / (2 rho_w) = g beta (T_w - T*) / 2 along y
    w = (slice(None), 0, slice(1, -1))
    assert np.allclose(g["u"][1][w], 0.5 * g["F"][1][w] / g["rho"][w], rtol=1e-12, atol=0)
    assert np.abs(g["u"][1][w]).min() > 1e-7


def test_energy_couette_matches_reference(orc):
    """The reference's ENERGY model (LBM.h:58) on its Couette case, D2Q9:
    temperature populations on the flow lattice with the cubic equilibrium
    (lbm.cpp:636-653), viscous heating with the F_vis history term
    (lbm.cpp:121-177), anti-bounce-back Dirichlet walls (lbm.cpp:277-280),
    T and q summed on every cell (lbm.cpp:776-792).  Summed in the
    reference's order: bit-exact after 2000 steps, ghosts included."""
    g = np.load(os.path.join(GOLDEN, "couette_energy_ny30_re20_2000.npz"))
    lat, c = orc.couette_energy(int(g["ny"]), float(g["Re"]))
    assert lat.step_plain(int(g["steps"])) == 0
    assert np.array_equal(lat.rho[1], g["rho"])
    assert np.array_equal(np.stack([lat.ux[1], lat.uy[1], lat.uz[1]]), g["u"])
    assert np.array_equal(lat.T[1], g["T"])
    assert np.array_equal(lat.hq[:, 1], g["q"])
    # the walls' temperature: Determine_Wall_Temperature's periodic neighbour
    # search (lbm.cpp:965-981) wraps each wall row onto the other, so both
    # ghost rows hold the mean of Tb and Tt from Init on (their g are never
    # streamed)
    mid = 0.5 * (c["Tb"] + c["Tt"])
    assert abs(g["T"][0, 1] - mid) < 1e-12 and abs(g["T"][-1, 1] - mid) < 1e-12
    # viscous heating lifts the centre above both walls
    assert g["T"][16, 1] > mid + 1e-4


@pytest.mark.parametrize("case", [("cylbasic", 100, 60, 20.0, 200.0, 0.1, 1), ("tandem", 160, 100, 10, 100.0, 0.05, 2),
                                  ("triangle", 100, 80, 10, 100.0, 0.05, 3)], ids=lambda c: c[0])
def test_staircase2d_matches_reference(orc, case):
    """The D2Q9 staircase bodies with momentum-exchange Cl/Cd: Cylinder_Basic,
    Cylinder_Tandem_Circle and Cylinder_Tandem_Triangle (lbm.cpp:1429-1757),
    their set-ups restated from the reference (cell types equal), MEA_CL /
    MEA_CD in each body's box (main.cpp:242-356) after every step."""
    kind, nx, ny, D, Re, u, nb = case
    g = np.load(os.path.join(GOLDEN, "staircase2d_%s_300.npz" % kind))
    lat, cl, cd = orc.staircase2d_run(kind, nx, ny, D, Re, u, int(g["steps"]), 1.5, nb)
    assert np.array_equal(lat.types[1], g["types"])
    scale = np.abs(g["cd"]).max()
    assert np.abs(cl - g["cl"]).max() < 1e-12 * scale and np.abs(cd - g["cd"]).max() < 1e-12 * scale
    f = np.stack([lat.rho[1], lat.ux[1], lat.uy[1]])
    wr, wc = g["wrows"], g["wcols"]
    assert np.abs(f[:, wr[0]:wr[1], wc[0]:wc[1]] - g["window"]).max() < 1e-13
    assert np.allclose(f.reshape(3, -1).sum(axis=1), g["sums"], rtol=1e-12, atol=1e-10)


@pytest.mark.parametrize("energy", [False, True], ids=["plain", "energy"])
def test_poiseuille_matches_reference(orc, energy):
    """The reference's Poiseuille_Flow build (lbm.cpp:1495-1535): the body
    force -dp/dx set on the fluid at set-up and on every cell in each
    MacroProp (lbm.cpp:800-801), so the walls report u = F/2 from the
    second MacroProp on and bounce back as moving walls; with ENERGY also the
    Dirichlet walls at T = 1 and the viscous heating.  Bit-exact after 1500
    steps, ghosts included."""
    g = np.load(os.path.join(GOLDEN, "poiseuille_ny30_re20%s_1500.npz" % ("_energy" if energy else "")))
    lat, c = orc.poiseuille(int(g["ny"]), float(g["Re"]), energy=energy)
    assert lat.step_plain(int(g["steps"])) == 0
    assert np.array_equal(lat.rho[1], g["rho"])
    assert np.array_equal(np.stack([lat.ux[1], lat.uy[1], lat.uz[1]]), g["u"])
    # the wall rows move at F / 2
    assert np.all(g["u"][0, 0] == 0.5 * c["fx"]) or np.allclose(g["u"][0, 0], 0.5 * c["fx"], rtol=1e-12)
    if energy:
        assert np.array_equal(lat.T[1], g["T"])
        assert np.array_equal(lat.hq[:, 1], g["q"])
