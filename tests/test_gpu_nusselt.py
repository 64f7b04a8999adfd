"""Find_Nusselt_number (lbm.cpp:3538-3561) on the device, lbmgpu_nusselt:
the FP64 fixed-order reduction against the same sum over the handle's own
moments (agreement to 1e-12 of Nu - 1), on a D3Q7 Rayleigh-Benard box with
an interior solid and on a D2Q9 ENERGY channel; and against the oracle's
restatement (orc_nusselt_volume) for the D2Q9 case, within the FP32 error of
u_y and T carried through the formula."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _numpy_nu(m, alpha, dT, Ny, fluid):
    return 1.0 + (m["uy"].astype(np.float64) * m["T"].astype(np.float64))[fluid].mean() / (alpha * dT / (Ny + 1))


def test_nusselt_d3q7_convection_box(pkg):
    n, ny, nz = 24, 16, 8
    Tb, Tt = 1.0, 0.0
    faces = {f: {"kind": pkg.FACE_WALL} for f in range(6)}
    faces[2] = {"kind": pkg.FACE_WALL, "thermal_kind": pkg.TWALL_DIRICHLET, "T": Tb}
    faces[3] = {"kind": pkg.FACE_WALL, "thermal_kind": pkg.TWALL_DIRICHLET, "T": Tt}
    tau_g = 0.8
    cfg = pkg.make_config(n, ny, nz, 0.7, "f32", faces, thermal=True, tau_g=tau_g, T_init=0.5, T_ref=0.5,
                          gbeta=(0.0, 2e-4, 0.0))
    s = pkg.Solver(cfg)
    mask = np.zeros((nz, ny, n), np.uint8)
    mask[2:5, 6:9, 10:13] = 1
    s.set_solids(mask)
    s.init()
    s.step(400)
    alpha = 0.25 * (tau_g - 0.5)
    nu_dev = s.nusselt(alpha, Tb - Tt)
    m = s.moments()
    ref = _numpy_nu(m, alpha, Tb - Tt, ny, mask == 0)
    assert abs(m["uy"]).max() > 1e-6
    assert abs(nu_dev - ref) < 1e-12 * max(1.0, abs(ref - 1.0)), (nu_dev, ref)


def test_nusselt_d2q9_energy_vs_oracle(pkg, orc):
    from test_gpu_energy import _solver

    ny, Re, steps = 24, 30.0, 300
    s, c = _solver(pkg, orc, ny, Re, nx=6, tau=0.8)
    s.step(steps)
    dT = c["Tt"] - c["Tb"]
    alpha = c["nu"] / 0.7
    nu_dev = s.nusselt(alpha, dT)
    m = s.moments()
    assert nu_dev == pytest.approx(_numpy_nu({"uy": m["uy"], "T": m["T"]}, alpha, dT, ny, np.ones_like(m["T"], bool)),
                                   rel=1e-14, abs=1e-14)
    lat, _ = orc.couette_energy(ny, Re, tau=0.8, nx=6)
    lat.step_plain(steps)
    nu_orc = lat.L.orc_nusselt_volume(lat.h, alpha, dT)
    # u_y vanishes in this parallel flow but for rounding, which the small
    # alpha dT / (Ny + 1) magnifies: the two may differ by at most the FP32
    # u_y error carried through the formula
    duy = np.abs(m["uy"][0].astype(np.float64) - lat.uy[1, 1:-1, :]).max()
    dT_err = np.abs(m["T"][0].astype(np.float64) - lat.T[1, 1:-1, :]).max()
    bound = (duy * lat.T.max() + dT_err * np.abs(lat.uy).max()) / (alpha * dT / (ny + 1))
    assert abs(nu_dev - nu_orc) <= 1.01 * bound + 1e-12, (nu_dev, nu_orc, bound)
