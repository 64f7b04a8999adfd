"""Host-side checks of the C ABI that need no GPU: the library loads, exports
every entry point include/lbmgpu.h declares, maps the reference's per-cell
geometry to face descriptors, and fails loudly (status codes, never a
crash) when no device is usable."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    txt = open(os.path.join(ROOT, "include", "lbmgpu.h")).read()
    return sorted(set(re.findall(r"\b(lbmgpu_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol(pkg):
    L = pkg.load()
    declared = _declared()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(pkg.ABI_SYMBOLS) == declared
    assert L.lbmgpu_abi_version() == 3


def _ref_geometry(nx, ny, nz):
    NX, NY, NZ = nx + 2, ny + 2, nz + 2
    t = np.zeros((NZ, NY, NX), np.uint8)
    z = np.zeros((NZ, NY, NX))
    return t, z.copy(), z.copy(), z.copy(), z.copy()


def test_config_from_types_cavity(pkg):
    t, rho, ux, uy, uz = _ref_geometry(8, 6, 5)
    rho[:] = 1.0
    t[:] = 1
    t[1:-1, 1:-1, 1:-1] = 0
    ux[:, -1, :] = 0.05  # lid plane j = Ny+1
    cfg = pkg.config_from_types(8, 6, 5, 0.8, t, rho, ux, uy, uz)
    assert (cfg.nx, cfg.ny, cfg.nz) == (8, 6, 5)
    assert [cfg.faces[f].kind for f in range(6)] == [pkg.FACE_WALL] * 6
    assert cfg.faces[3].u[0] == 0.05 and cfg.faces[2].u[0] == 0.0


def test_config_from_types_channel_and_periodic(pkg):
    # Sphere_BB / IBM style: TYPE_IN at x=0, TYPE_OUT elsewhere on the ghosts
    t, rho, ux, uy, uz = _ref_geometry(10, 6, 6)
    rho[:] = 1.0
    ux[:] = 0.1
    t[:, :, 0] = 3
    t[:, :, -1] = 2
    t[:, 0, 1:-1] = 2
    t[:, -1, 1:-1] = 2
    t[0, 1:-1, 1:-1] = 2
    t[-1, 1:-1, 1:-1] = 2
    cfg = pkg.config_from_types(10, 6, 6, 0.6, t, rho, ux, uy, uz)
    assert cfg.faces[0].kind == pkg.FACE_INLET and cfg.faces[1].kind == pkg.FACE_OUTLET_EQ
    assert cfg.faces[0].u[0] == 0.1
    # Couette style (lbm.cpp:1537-1555): TYPE_F ghosts in x and z wrap over N+2
    t, rho, ux, uy, uz = _ref_geometry(2, 12, 2)
    rho[:] = 1.0
    t[:, 0, :] = 1
    t[:, -1, :] = 1
    ux[:, -1, :] = 0.02
    cfg = pkg.config_from_types(2, 12, 2, 0.9, t, rho, ux, uy, uz)
    assert (cfg.nx, cfg.ny, cfg.nz) == (4, 12, 4)
    assert cfg.faces[0].kind == pkg.FACE_PERIODIC and cfg.faces[4].kind == pkg.FACE_PERIODIC
    assert cfg.faces[3].kind == pkg.FACE_WALL and cfg.faces[3].u[0] == 0.02


def test_config_from_types_interior_solids(pkg):
    """Interior solid cells at rest are accepted (their mask goes to
    lbmgpu_set_solids); a moving one or another interior type is refused."""
    t, rho, ux, uy, uz = _ref_geometry(6, 6, 6)
    t[:] = 1
    t[1:-1, 1:-1, 1:-1] = 0
    t[3, 3, 3] = 1
    cfg = pkg.config_from_types(6, 6, 6, 0.8, t, rho, ux, uy, uz)
    assert (cfg.nx, cfg.ny, cfg.nz) == (6, 6, 6)
    ux2 = ux.copy()
    ux2[3, 3, 3] = 0.01
    with pytest.raises(pkg.LbmError) as e:
        pkg.config_from_types(6, 6, 6, 0.8, t, rho, ux2, uy, uz)
    assert e.value.status == 7
    t[3, 3, 3] = 3
    with pytest.raises(pkg.LbmError) as e:
        pkg.config_from_types(6, 6, 6, 0.8, t, rho, ux, uy, uz)
    assert e.value.status == 7


def test_create_rejects_bad_config_without_touching_device(pkg):
    cfg = pkg.cavity_config(8, tau=0.5)
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(cfg)
    assert e.value.status == 1
    cfg = pkg.cavity_config(8)
    cfg.faces[0].kind = pkg.FACE_PERIODIC
    with pytest.raises(pkg.LbmError):
        pkg.Solver(cfg)


def test_output_csv_reference_format(pkg, tmp_path):
    """OutputCSV (lbm.cpp:3169-3186): header "time,error", time (i+1) dt."""
    p = str(tmp_path / "cd.csv")
    pkg.output_csv(p, [1.5, 0.25, 3e-7], 0.5)
    assert open(p).read() == "time,error\n0.5,1.5\n1,0.25\n1.5,3e-07\n"


def test_more_details_entry_points_reject_null_handles(pkg):
    """The MORE_DETAILS calls check their arguments before any device work."""
    L = pkg.load()
    assert L.lbmgpu_set_more_details(None, 1) == 1
    assert L.lbmgpu_sup_macroprop(None, 10, 10, 1.0) == 1
    assert L.lbmgpu_download_details(None, None) == 1
    assert L.lbmgpu_download_stats(None, None, None, None) == 1
    assert L.lbmgpu_output_avg_vtk(None, b"x.vtr", 0.1, None) == 1
    assert "null" in L.lbmgpu_last_error().decode() or "bad argument" in L.lbmgpu_last_error().decode()


def test_config_energy_2d_maps_couette_and_refuses_the_rest(pkg):
    """lbmgpu_config_energy_2d: main_setup_Couette's type_Energy / T set-up
    (lbm.cpp:1552-1572) -> Dirichlet wall faces; the unsupported energy
    set-ups fail with LBM_ERR_UNSUPPORTED before any device work."""
    nx, ny = 2, 10
    t = np.zeros((ny + 2, nx + 2), np.uint8)
    t[0] = t[-1] = 1
    te = np.zeros_like(t)
    te[0] = te[-1] = 6
    T = np.full(t.shape, 0.5)
    T[-1] = 0.625
    cfg = pkg.config_energy_2d(pkg.config_from_types_2d(nx, ny, 0.9, t), nx, ny, t, te, T, 0.8, 2.0)
    assert cfg.thermal == pkg.THERMAL_ENERGY and cfg.cp == 2.0 and cfg.tau_g == 0.8 and cfg.T_init == 0.5
    assert [cfg.faces[f].thermal_kind for f in (2, 3)] == [pkg.TWALL_DIRICHLET] * 2
    assert (cfg.faces[2].T, cfg.faces[3].T) == (0.5, 0.625)
    # TYPE_Q: a Neumann wall (j.n = 0); any other type_Energy: adiabatic;
    # both keep their set-up T
    for top, kind in ((7, pkg.TWALL_NEUMANN), (0, pkg.TWALL_ADIABATIC)):
        te2 = te.copy()
        te2[-1] = top
        c2 = pkg.config_energy_2d(pkg.config_from_types_2d(nx, ny, 0.9, t), nx, ny, t, te2, T, 0.8, 2.0)
        assert (c2.faces[2].thermal_kind, c2.faces[3].thermal_kind) == (pkg.TWALL_DIRICHLET, kind)
        assert (c2.faces[2].T, c2.faces[3].T) == (0.5, 0.625)
    for bad_te, bad_T, word in ((7, None, "mixes"), (0, None, "mixes"), (6, "fluid", "uniform")):
        te2 = te.copy()
        te2[0, 2] = bad_te
        T2 = T.copy()
        if bad_T:
            T2[3, 1] = 0.51
        with pytest.raises(pkg.LbmError) as e:
            pkg.config_energy_2d(pkg.config_from_types_2d(nx, ny, 0.9, t), nx, ny, t, te2, T2, 0.8, 2.0)
        assert e.value.status == 7 and word in str(e.value), (word, str(e.value))
    # an inlet face
    t3 = t.copy()
    t3[1:-1, 0] = 3
    t3[1:-1, -1] = 2
    with pytest.raises(pkg.LbmError) as e:
        pkg.config_energy_2d(pkg.config_from_types_2d(nx, ny, 0.9, t3), nx, ny, t3, te, T, 0.8, 2.0)
    assert e.value.status == 7
    # Neumann walls are a D2Q9 ENERGY option; ENERGY on D3Q19 is lbm_energy3d
    c3 = pkg.channel_config(8, 8, 8, 0.8)
    c3.faces[2].thermal_kind = pkg.TWALL_NEUMANN
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(c3)
    assert e.value.status == 7 and "Neumann" in str(e.value)
    c4 = pkg.channel_config(8, 8, 8, 0.8)
    c4.thermal, c4.tau_g, c4.cp = pkg.THERMAL_ENERGY, 0.8, 2.0
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(c4)
    assert e.value.status == 7 and "energy3d" in str(e.value)
    c4.thermal = 5
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(c4)
    assert e.value.status == 1
    # create: the D3Q7 model is not a D2Q9 option; ENERGY needs cp > 0
    c2 = pkg.config_from_types_2d(nx, ny, 0.9, t)
    c2.thermal, c2.tau_g = pkg.THERMAL_D3Q7, 0.8
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(c2)
    assert e.value.status == 7
    cfg.storage = pkg.STORAGE["f16"]
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(cfg)
    assert e.value.status == 7 and "FP32" in str(e.value)
    cfg.storage = pkg.STORAGE["f32"]
    cfg.cp = 0.0
    with pytest.raises(pkg.LbmError) as e:
        pkg.Solver(cfg)
    assert e.value.status == 1


def test_ctypes_mirrors_match_the_header_layouts(pkg, tmp_path):
    """Every public struct of include/lbmgpu.h has the size and field offsets
    of its ctypes mirror in the package, as a C compiler lays it out."""
    import ctypes as C
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"lbm_face": pkg.Face, "lbm_config": pkg.Config, "lbm_ibm_config": pkg.IbmConfig,
               "lbm_serve_request": pkg.ServeRequest, "lbm_serve_options": pkg.ServeOptions,
               "lbm_serve_result": pkg.ServeResult, "lbm_energy3d_setup": pkg.Energy3DSetup}
    txt = open(os.path.join(ROOT, "include", "lbmgpu.h")).read()
    assert sorted(mirrors) == sorted(re.findall(r"typedef struct (lbm_\w+) \{", txt))
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "lbmgpu.h"', "int main(void) {"]
    expect = []
    for name, cls in mirrors.items():
        lines.append('    printf("%%zu\\n", sizeof(%s));' % name)
        expect.append(("sizeof " + name, C.sizeof(cls)))
        for field, _ in cls._fields_:
            lines.append('    printf("%%zu\\n", offsetof(%s, %s));' % (name, field))
            expect.append((name + "." + field, getattr(cls, field).offset))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)], text=True).split()]
    assert len(got) == len(expect)
    for (what, want), have in zip(expect, got):
        assert have == want, (what, have, want)
