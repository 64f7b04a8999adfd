"""GPU parity for the D2Q9 build (the reference's #define D2Q9, Nz = 1):
D2Q9 collide-stream with its boundary classes against the FP64 oracle, and
the two-dimensional IBM cylinders -- the shipped default (implicit
multi-direct forcing), the explicit scheme and the transversely oscillating
body -- against the reference's own runs (tests/golden).

Tolerances: FP32 fields within 1e-5 of the reference velocity (3e-5 for the
staircase bodies at tau = 0.53); MEA Cl and Cd within 2e-5 of max |Cd|; Cl and Cd of
the IBM cylinders within 2e-6 of the largest |Cd| of the run (measured: 7.0e-8
implicit, 1.1e-7 explicit, 3.9e-7 oscillating; the force sums run over FP32
velocities); FP16 storage within 1e-3 (measured 2.4e-4)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CX9 = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY9 = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])


def _layer_moments(lat, xs=slice(1, -1), body=(0.0, 0.0)):
    """rho, u = (sum f c + F/2) / rho of the oracle's computational layer
    k = 1, interior rows, columns xs."""
    f = lat.f[:, 1, 1:-1, xs]
    rho = f.sum(axis=0)
    ux = (np.tensordot(CX9, f, axes=(0, 0)) + 0.5 * body[0]) / rho
    uy = (np.tensordot(CY9, f, axes=(0, 0)) + 0.5 * body[1]) / rho
    return rho, ux, uy


def _check_fields(m, rho, ux, uy, uref, tol=1e-5):
    e = max(np.abs(m["ux"][0] - ux).max(), np.abs(m["uy"][0] - uy).max()) / uref
    er = np.abs(m["rho"][0] - rho).max()
    assert e < tol and er < tol, (e, er)
    assert not np.any(m["uz"])
    return e


def test_d2q9_cavity_vs_oracle(pkg, orc):
    nx, ny, tau, lid, steps = 48, 32, 0.7, 0.05, 400
    lat = orc.Lattice(9, nx, ny, 1, tau)
    t = lat.types
    t[:] = orc.TYPE_S
    t[:, 1:-1, 1:-1] = orc.TYPE_F
    lat.ux[:, -1, :] = lid
    lat.init()
    cfg = pkg.config_from_types_2d(nx, ny, tau, t[1], lat.rho[1], lat.ux[1], lat.uy[1])
    assert cfg.lattice == pkg.LATTICE_D2Q9 and cfg.nz == 1
    s = pkg.Solver(cfg)
    s.init()
    s.step(steps)
    assert s.status() == 0
    lat.step_plain(steps)
    _check_fields(s.moments(), *_layer_moments(lat), lid)


def test_d2q9_poiseuille_periodic_forced_vs_oracle(pkg, orc):
    """Periodic in x over the Nx + 2 columns (TYPE_F ghosts), walls in y,
    a uniform body force (MacroProp's F/2 shift, Guo source)."""
    nx, ny, tau, steps, fx = 6, 24, 0.9, 600, 2e-6
    lat = orc.Lattice(9, nx, ny, 1, tau)
    t = lat.types
    t[:] = orc.TYPE_F
    t[:, 0, :] = orc.TYPE_S
    t[:, -1, :] = orc.TYPE_S
    lat.init()
    lat.set_body_force(fx, 0.0, 0.0)
    # main_setup_Poiseuille sets F = -dp/dx at set-up (lbm.cpp:1518), so the
    # first collision is forced too
    lat.Fx[t == orc.TYPE_F] = fx
    cfg = pkg.config_from_types_2d(nx, ny, tau, t[1], lat.rho[1], lat.ux[1], lat.uy[1])
    assert (cfg.nx, cfg.ny) == (nx + 2, ny)
    cfg.body_force[0] = fx
    s = pkg.Solver(cfg)
    s.init()
    s.step(steps)
    lat.step_plain(steps)
    rho, ux, uy = _layer_moments(lat, xs=slice(None), body=(fx, 0.0))
    umax = np.abs(ux).max()
    assert umax > 1e-4
    _check_fields(s.moments(), rho, ux, uy, umax)


def _cylinder_gpu(pkg, orc, g, steps, storage="f32", graph_steps=0, **kw):
    s, u_max, area = _cylinder_solver(pkg, orc, g, storage, graph_steps, **kw)
    s.step(steps)
    assert s.status() == 0
    rows = s.forces()
    assert rows.shape[0] == steps and np.array_equal(rows[:, 7], np.arange(1, steps + 1))
    q = 0.5 * u_max ** 2 * area
    return s, rows[:, 1] / q, rows[:, 0] / q


def _cylinder_solver(pkg, orc, g, storage="f32", graph_steps=0, **kw):
    """The reference's cylinder set-up (main_setup_Cylinder_IBM and its
    variants) on a fresh D2Q9 handle, markers registered, not stepped;
    returns the solver, u_max and the Cl/Cd reference length."""
    nx, ny, D, nodes = int(g["nx"]), int(g["ny"]), float(g["D"]), int(g["nodes"])
    u_max, Re = kw.pop("u_max", 0.1), kw.pop("Re", 40.0)
    marker_dy = kw.pop("marker_dy", 0.0)
    ibm_overlap = kw.pop("ibm_overlap", 0)
    at_rest, center, area = kw.pop("at_rest", False), kw.pop("center", None), kw.pop("area", D)
    tau = 0.5 + (u_max * D / Re) / (1.0 / 3.0)
    t = np.zeros((ny + 2, nx + 2), np.uint8)
    t[:, 0] = orc.TYPE_OUT if at_rest else orc.TYPE_IN
    t[:, -1] = orc.TYPE_OUT
    t[0, :] = orc.TYPE_OUT
    t[-1, :] = orc.TYPE_OUT
    ones = np.ones((ny + 2, nx + 2))
    u0 = 0.0 if at_rest else u_max
    cfg = pkg.config_from_types_2d(nx, ny, tau, t, ones, u0 * ones, 0.0 * ones)
    cfg.storage = pkg.STORAGE[storage]
    cfg.graph_steps = graph_steps
    cfg.ibm_overlap = ibm_overlap
    cfg.u0[0] = u0
    s = pkg.Solver(cfg)
    s.init()
    cx, cy = (nx / 5.0, ny / 2.0) if center is None else center
    mk = orc.cylinder_markers_literal(nodes, D, cx, cy + marker_dy)
    xyz = np.stack([mk["x"], mk["y"], mk["z"]])
    nrm = np.stack([mk["nx"], mk["ny"], mk["nz"]])
    vsolid = kw.pop("vsolid", orc.REF_PI * D * D * 0.25)
    s.set_markers(xyz, mk["ds"], D / 2.0, (cx, cy, 1.0), literal_sign=True, normals=nrm, rho_nearest=True,
                  added_mass=True, volume=vsolid, **kw)
    return s, u_max, area


def _coeff_err(cl, cd, g):
    scale = np.abs(g["cd"]).max()
    return max(np.abs(cd - g["cd"]).max(), np.abs(cl - g["cl"]).max()) / scale


def test_d2q9_ibm_cylinder_vs_reference(pkg, orc):
    """The shipped default case (Cylinder_IBM, implicit forcing, literal force
    sign, nearest-node density, added mass), shrunk: Cl / Cd after every step
    against the reference's run, the fields against the oracle (pinned to the
    same run)."""
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    steps = int(g["steps"])
    s, cl, cd = _cylinder_gpu(pkg, orc, g, steps, m_max=int(g["m_max"]))
    e = _coeff_err(cl, cd, g)
    print("cylinder Cl/Cd error / max|Cd|: %.3g" % e)
    assert e < 2e-6
    lat, mk, _, _ = orc.cylinder2d_literal(80, 40, 10.0, 40, int(g["m_max"]), steps)
    _check_fields(s.moments(), *_layer_moments(lat), 0.1)


def test_d2q9_ibm_explicit_vs_reference(pkg, orc):
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_explicit_100.npz"))
    s, cl, cd = _cylinder_gpu(pkg, orc, g, int(g["steps"]), m_max=1, scheme=1)
    e = _coeff_err(cl, cd, g)
    print("explicit Cl/Cd error / max|Cd|: %.3g" % e)
    assert e < 2e-6
    lat, _, _, _ = orc.cylinder2d_literal(80, 40, 10.0, 40, 1, int(g["steps"]), scheme=1)
    _check_fields(s.moments(), *_layer_moments(lat), 0.1)


def test_d2q9_ibm_transverse_oscillation_vs_reference(pkg, orc):
    """Moving markers and box (V_CM(t) of Cylinder_Transverse_Oscillation),
    the added mass of a changing V_CM, markers at center_y + amplitude."""
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_transverse_100.npz"))
    D = float(g["D"])
    s, cl, cd = _cylinder_gpu(pkg, orc, g, int(g["steps"]), m_max=5, u_max=0.05, Re=100.0, marker_dy=2.0,
                              vsolid=orc.REF_PI * D * D * 0.25 * 3, motion=pkg.MOTION_TRANSVERSE_OSC,
                              motion_amp=2.0, motion_freq=0.005)
    e = _coeff_err(cl, cd, g)
    print("transverse Cl/Cd error / max|Cd|: %.3g" % e)
    assert e < 2e-6
    assert np.abs(s.markers().reshape(3, -1)[1] - g["markers"][:, 1]).max() < 1e-12
    body = s.body()
    lat, mk, _, _ = orc.cylinder2d_literal(80, 40, D, 40, 5, int(g["steps"]), u_max=0.05, Re=100.0,
                                           motion=orc.transverse_motion(2.0, 0.005),
                                           vsolid=orc.REF_PI * D * D * 0.25 * 3, marker_dy=2.0)
    _check_fields(s.moments(), *_layer_moments(lat), 0.05)
    # the body's V_CM of the last step
    assert abs(body[4] - orc.transverse_motion(2.0, 0.005)(float(g["steps"]))[1]) < 1e-15


@pytest.mark.parametrize("case", ["inline", "towed"])
def test_d2q9_ibm_moving_in_fluid_at_rest_vs_reference(pkg, orc, case):
    """The inline oscillation (V_x = -u cos 2 pi f t, Cd over D + dx) and
    the towed cylinder (V_x = -u), both in fluid at rest with TYPE_OUT on
    every face: Cl / Cd after every step, the markers and the fields against
    the reference's runs.  The step-1 added-mass impulse dominates max |Cd|;
    the later steps are held to their own scale too."""
    from test_oracle_golden import moving_case_kwargs

    name = "cylinder80x40_D10_n40_m5_inline_100.npz" if case == "inline" else "cylinder120x40_D10_n40_m5_towed_100.npz"
    g = np.load(os.path.join(GOLDEN, name))
    D, steps = float(g["D"]), int(g["steps"])
    okw = moving_case_kwargs(orc, case, D)
    kw = dict(m_max=5, u_max=okw["u_max"], Re=okw["Re"], at_rest=True, center=okw["center"],
              area=okw.get("area", D))
    if case == "inline":
        kw.update(vsolid=okw["vsolid"], motion=pkg.MOTION_INLINE_OSC, motion_amp=okw["u_max"], motion_freq=1e-3)
    else:
        kw.update(motion=pkg.MOTION_CONSTANT, velocity=(-0.1, 0.0, 0.0))
    s, cl, cd = _cylinder_gpu(pkg, orc, g, steps, **kw)
    e = _coeff_err(cl, cd, g)
    late = max(np.abs(cd - g["cd"])[1:].max(), np.abs(cl - g["cl"])[1:].max()) / np.abs(g["cd"][1:]).max()
    print("%s Cl/Cd error / max|Cd|: %.3g (steps 2.. on their own scale: %.3g)" % (case, e, late))
    assert e < 2e-6 and late < 2e-5
    mk = s.markers().reshape(3, -1)
    assert np.abs(mk[0] - g["markers"][:, 0]).max() < 1e-12
    lat, _, _, _ = orc.cylinder2d_literal(int(g["nx"]), int(g["ny"]), D, int(g["nodes"]), steps=steps, **okw)
    _check_fields(s.moments(), *_layer_moments(lat), okw["u_max"])


def test_d2q9_ibm_fp16_storage(pkg, orc):
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    _, cl, cd = _cylinder_gpu(pkg, orc, g, int(g["steps"]), storage="f16", m_max=int(g["m_max"]))
    e = _coeff_err(cl, cd, g)
    print("cylinder FP16 Cl/Cd error / max|Cd|: %.3g" % e)
    assert e < 1e-3


def test_d2q9_graph_replay_matches_eager(pkg, orc):
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    out = []
    for gs in (8, -1):
        s, cl, cd = _cylinder_gpu(pkg, orc, g, 41, graph_steps=gs, m_max=3)
        out.append((s.moments(), cl, cd))
    for c in ("rho", "ux", "uy"):
        assert np.array_equal(out[0][0][c], out[1][0][c]), c
    assert np.array_equal(out[0][1], out[1][1]) and np.array_equal(out[0][2], out[1][2])


@pytest.mark.parametrize("graph_steps", [8, -1], ids=["graphs", "eager"])
def test_d2q9_split_streams_match_serial_order(pkg, orc, graph_steps):
    """A fixed body's step split across two streams (near box and IBM on
    one, the far region on the other) gives the same bits as the serial
    order: the far region never reads what the IBM phase writes."""
    g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
    out = []
    for ov in (0, -1):
        s, cl, cd = _cylinder_gpu(pkg, orc, g, 41, graph_steps=graph_steps, m_max=3, ibm_overlap=ov)
        out.append((s.moments(), cl, cd, s.markers()))
    for c in ("rho", "ux", "uy"):
        assert np.array_equal(out[0][0][c], out[1][0][c]), c
    for i in (1, 2, 3):
        assert np.array_equal(out[0][i], out[1][i])


def test_d2q9_unsupported_calls_fail_loudly(pkg, tmp_path):
    t = np.ones((10, 12), np.uint8)
    t[1:-1, 1:-1] = 0
    s = pkg.Solver(pkg.config_from_types_2d(10, 8, 0.8, t))
    s.init()
    for call in (lambda: s.solid_forces(),):
        with pytest.raises(pkg.LbmError) as e:
            call()
        assert e.value.status == 7
    # solid cells go in before init; markers and solids do not mix
    with pytest.raises(pkg.LbmError) as e:
        s.set_solids(np.zeros((1, 8, 10)))
    assert e.value.status == 6
    s2 = pkg.Solver(pkg.config_from_types_2d(10, 8, 0.8, t))
    m = np.zeros((1, 8, 10))
    m[0, 3:5, 3:5] = 1
    s2.set_solids(m)
    with pytest.raises(pkg.LbmError) as e:
        s2.set_markers(np.zeros((3, 4)), np.ones(4), 1.0, (5.0, 4.0, 1.0))
    assert e.value.status == 7
    # MORE_DETAILS and markers do not mix on D2Q9 handles (the reference's IBM
    # loop never calls MacroProp, which forms the details), in either order
    s3 = pkg.Solver(pkg.config_from_types_2d(10, 8, 0.8, t))
    s3.init()
    s3.set_markers(np.zeros((3, 4)) + np.array([[5.0], [4.0], [1.0]]), np.ones(4), 1.0, (5.0, 4.0, 1.0))
    with pytest.raises(pkg.LbmError) as e:
        s3.set_more_details(True)
    assert e.value.status == 7
    s4 = pkg.Solver(pkg.config_from_types_2d(10, 8, 0.8, t))
    s4.init()
    s4.set_more_details(True)
    with pytest.raises(pkg.LbmError) as e:
        s4.set_markers(np.zeros((3, 4)) + np.array([[5.0], [4.0], [1.0]]), np.ones(4), 1.0, (5.0, 4.0, 1.0))
    assert e.value.status == 7


STAIRCASE = [("cylbasic", 100, 60, 20.0, 200.0, 0.1, 1), ("tandem", 160, 100, 10, 100.0, 0.05, 2),
             ("triangle", 100, 80, 10, 100.0, 0.05, 3)]


def _staircase_gpu(pkg, orc, case, storage="f32"):
    kind, nx, ny, D, Re, u, nb = case
    lat, boxes, area = orc.staircase2d(kind, nx, ny, D, Re, u, 1.5, nb)
    t = lat.types[1].copy()
    solid = t[1:-1, 1:-1] == orc.TYPE_S
    t[1:-1, 1:-1][solid] = orc.TYPE_F
    rho, ux, uy = lat.rho[1], lat.ux[1], lat.uy[1]
    cfg = pkg.config_from_types_2d(nx, ny, lat.tau, t, rho, ux, uy)
    assert (cfg.nx, cfg.ny) == (nx, ny)
    cfg.storage = pkg.STORAGE[storage]
    s = pkg.Solver(cfg)
    s.set_solids(solid[None].astype(np.uint8))
    z = np.zeros((1, ny, nx))
    s.init((rho[None, 1:-1, 1:-1], ux[None, 1:-1, 1:-1], uy[None, 1:-1, 1:-1], z))
    return s, lat, boxes, 0.5 * u * u * area


@pytest.mark.parametrize("case", STAIRCASE, ids=lambda c: c[0])
def test_d2q9_staircase_mea_vs_reference(pkg, orc, case):
    """Staircase bodies on a D2Q9 handle (Cylinder_Basic and the tandem
    circles / triangles): MEA_CL / MEA_CD of every body in its own box after
    every step against the reference's runs; the fields against the oracle
    (pinned to the same runs)."""
    g = np.load(os.path.join(GOLDEN, "staircase2d_%s_300.npz" % case[0]))
    steps = int(g["steps"])
    s, lat, boxes, q = _staircase_gpu(pkg, orc, case)
    nb = len(boxes)
    cl, cd = np.zeros((nb, steps)), np.zeros((nb, steps))
    for k in range(steps):
        s.step(1)
        for b, box in enumerate(boxes):
            F = s.mea_box(tuple(box) + (1, 1))
            cd[b, k] = F[0] / q
            cl[b, k] = -F[1] / q
    assert s.status() == 0
    scale = np.abs(g["cd"]).max()
    e = max(np.abs(cd - g["cd"]).max(), np.abs(cl - g["cl"]).max()) / scale
    print("%s MEA Cl/Cd error / max|Cd|: %.3g" % (case[0], e))
    assert e < 2e-5
    lat.step_plain(steps)
    m = s.moments()
    fluid = lat.types[1, 1:-1, 1:-1] != orc.TYPE_S
    u = case[5]
    # tau = 0.53 for Cylinder_Basic: FP32 fields within 3e-5 u (measured 1.1e-5)
    for c, r in (("ux", lat.ux), ("uy", lat.uy)):
        err = np.abs(m[c][0] - r[1, 1:-1, 1:-1])[fluid].max() / u
        print("%s %s error / u: %.3g" % (case[0], c, err))
        assert err < 3e-5, c
    assert np.abs(m["rho"][0] - lat.rho[1, 1:-1, 1:-1]).max() < 1e-5
    # solid cells keep their set-up equilibrium: rho = 1, u = 0
    assert np.all(m["ux"][0][~fluid] == 0) and np.allclose(m["rho"][0][~fluid], 1.0, atol=1e-6)


def test_d2q9_staircase_graph_replay_and_fp16(pkg, orc):
    """Graph replay equals eager stepping bit for bit with solid cells; FP16
    storage keeps the tandem circles' Cd within 1e-2 of the FP32 run
    (measured 3.4e-3: the exchange sums stored populations near the walls,
    each with FP16's 1e-5 rounding)."""
    case = STAIRCASE[1]
    out = []
    for storage in ("f32", "f16"):
        s, lat, boxes, q = _staircase_gpu(pkg, orc, case, storage)
        s.step(200)
        out.append(np.array([s.mea_box(tuple(b) + (1, 1))[0] / q for b in boxes]))
    assert np.abs(out[1] - out[0]).max() < 1e-2 * np.abs(out[0]).max()
    fields = []
    for gs in (8, -1):
        lat, boxes, area = orc.staircase2d(*case[:6], 1.5, case[6])
        t = lat.types[1].copy()
        solid = t[1:-1, 1:-1] == orc.TYPE_S
        t[1:-1, 1:-1][solid] = orc.TYPE_F
        cfg = pkg.config_from_types_2d(case[1], case[2], lat.tau, t, lat.rho[1], lat.ux[1], lat.uy[1])
        cfg.graph_steps = gs
        s = pkg.Solver(cfg)
        s.set_solids(solid[None].astype(np.uint8))
        s.init()
        s.step(37)
        fields.append((s.moments()["ux"], s.mea_box(tuple(boxes[0]) + (1, 1))))
    assert np.array_equal(fields[0][0], fields[1][0]) and np.array_equal(fields[0][1], fields[1][1])


def test_d2q9_ibm_large_box_vs_oracle(pkg, orc):
    """A body large enough that its IBM box (67 x 67 nodes) leaves the
    register-resident pass for the shared-memory one."""
    nx, ny, D, nodes, mm, steps = 200, 120, 32.0, 100, 3, 12

    class G(dict):
        pass

    g = G(nx=nx, ny=ny, D=D, nodes=nodes)
    s, cl, cd = _cylinder_gpu(pkg, orc, g, steps, m_max=mm)
    lat, mk, rcl, rcd = orc.cylinder2d_literal(nx, ny, D, nodes, mm, steps)
    scale = np.abs(rcd).max()
    e = max(np.abs(cd - rcd).max(), np.abs(cl - rcl).max()) / scale
    print("large-box Cl/Cd error / max|Cd|: %.3g" % e)
    assert e < 2e-6
    _check_fields(s.moments(), *_layer_moments(lat), 0.1)


@pytest.mark.parametrize("case", ["cylinder", "staircase"])
def test_d2q9_split_step_calls_match_one_call(pkg, orc, case):
    """Graphs replay for whichever buffer a call starts from: 30 + 30 steps
    (the first call ends on the other buffer than its graph started from)
    equal 60 steps in one call, bit for bit."""
    def make():
        if case == "cylinder":
            g = np.load(os.path.join(GOLDEN, "cylinder80x40_D10_n40_m5_100.npz"))
            return _cylinder_solver(pkg, orc, g, m_max=int(g["m_max"]))[0]
        return _staircase_gpu(pkg, orc, STAIRCASE[1])[0]

    a, b = make(), make()
    a.step(30)
    a.step(30)
    b.step(60)
    ma, mb = a.moments(), b.moments()
    for c in ma:
        assert np.array_equal(ma[c], mb[c]), c
    if case == "cylinder":
        assert np.array_equal(a.forces(), b.forces())
