"""The fused step with several x-cells per thread (k_stepv: one 4-, 8- or
16-byte access per population row segment, warp shuffles for the x-shifted
links, the packed FP32 pair instructions for the arithmetic) against the
one-cell-per-thread kernel (k_step).  Both run the same explicitly rounded
arithmetic on the same pulled values, so every field must agree bit for
bit -- on walls, moving lids, inlets and outlets, periodic axes, body forces
and the D3Q7 thermal population, with rows a block spans exactly, rows
shorter than a warp and rows whose segment count is not a power of two."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(pkg, case, storage, cells):
    kw = {"storage": storage, "cells": cells}
    if case == "cavity64":
        return pkg.cavity_config(64, tau=0.7, lid=0.05, ny=24, nz=12, **kw)
    if case == "cavity96":
        return pkg.cavity_config(96, tau=0.7, lid=0.05, ny=20, nz=6, **kw)
    if case == "cavity40":
        return pkg.cavity_config(40, tau=0.6, lid=0.05, ny=16, nz=9, **kw)
    if case == "channel_zg":
        return pkg.channel_config(256, 20, 18, 0.56, u_in=0.05, **kw)
    if case == "channel_eq":
        return pkg.channel_config(64, 18, 10, 0.6, u_in=0.05, outlet=pkg.FACE_OUTLET_EQ, **kw)
    if case == "channel_thermal":
        return pkg.channel_config(64, 24, 10, 0.6, u_in=0.05, thermal=True, T_in=1.0, tau_g=0.7,
                                  gbeta=(0.0, 1e-4, 0.0), **kw)
    if case == "poiseuille_forced":
        faces = {0: {"kind": pkg.FACE_PERIODIC}, 1: {"kind": pkg.FACE_PERIODIC}}
        faces.update({f: {"kind": pkg.FACE_WALL} for f in (2, 3, 4, 5)})
        return pkg.make_config(64, 24, 8, 0.8, storage, faces, body=(1e-6, 0.0, 0.0), cells=cells)
    # periodic in x and z, moving wall on y+
    faces = {f: {"kind": pkg.FACE_PERIODIC} for f in (0, 1, 4, 5)}
    faces[2] = {"kind": pkg.FACE_WALL}
    faces[3] = {"kind": pkg.FACE_WALL, "u": (0.05, 0.0, 0.0)}
    return pkg.make_config(64, 24, 8, 0.7, storage, faces, cells=cells)


CASES = ["cavity64", "cavity96", "cavity40", "channel_zg", "channel_eq", "channel_thermal", "poiseuille_forced",
         "couette_xz"]
WIDTHS = {"f32": (2, 4), "f16": (2, 4, 8), "bf16": (2, 4, 8)}


def _run(pkg, cfg, steps=(1, 30, 19)):
    s = pkg.Solver(cfg)
    s.init()
    for n in steps:
        s.step(n)
    assert s.status() == 0
    m = s.moments()
    cells = s.cells_per_thread()
    s.close()
    return m, cells


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
@pytest.mark.parametrize("case", CASES)
def test_multicell_step_matches_single_cell_bitwise(pkg, case, storage):
    ref, c1 = _run(pkg, _case(pkg, case, storage, 1))
    assert c1 == 1
    for v in WIDTHS[storage]:
        if _case(pkg, case, storage, v).nx % v:
            continue
        got, cv = _run(pkg, _case(pkg, case, storage, v))
        assert cv == v, (case, storage, v, cv)
        for c in ref:
            assert np.array_equal(ref[c], got[c]), (case, storage, v, c)


def test_default_cells_per_thread(pkg):
    # two cells a thread for half storage on lattices of 2^20 cells or more
    for storage, v in (("f32", 1), ("f16", 2), ("bf16", 2)):
        s = pkg.Solver(pkg.cavity_config(128, tau=0.7, lid=0.05, ny=128, nz=64, storage=storage))
        assert s.cells_per_thread() == v, storage
        s.close()
    # smaller lattices sit in L2 and run one cell a thread
    s = pkg.Solver(pkg.cavity_config(64, tau=0.7, lid=0.05, ny=64, nz=64, storage="f16"))
    assert s.cells_per_thread() == 1
    s.close()
    # a row length that is not a multiple of the segment: one cell per thread
    s = pkg.Solver(pkg.cavity_config(31, tau=0.7, lid=0.05, ny=256, nz=256, storage="f16"))
    assert s.cells_per_thread() == 1
    s.close()


def test_multicell_sphere_matches_single_cell(pkg, orc):
    """The fixed IBM sphere with the near box carved out of the multi-cell far
    region (its x bounds rounded to whole segments): the same forces and
    fields as the one-cell-per-thread kernel, bit for bit (the spreading sums
    in fixed point, independent of the order of its atomics); with two cells
    a thread the moment export runs on the multi-cell kernel too, its band
    segments on the one-cell path."""
    nx, ny, nz, tau, D, nm, m_max, steps = 64, 40, 40, 0.53, 20.0, 1257, 5, 40
    center = (23.3, 20.2, 19.6)
    out = []
    for cells in (1, 2, 4):
        s = pkg.Solver(pkg.channel_config(nx, ny, nz, tau, u_in=0.05, storage="f32", cells=cells))
        s.init()
        mk = orc.fibonacci_sphere(nm, D, center)
        s.set_markers(np.stack([mk["x"], mk["y"], mk["z"]]), mk["ds"], D / 2.0, center, m_max=m_max)
        s.step(1)
        s.step(steps - 1)
        assert s.status() == 0
        out.append((s.forces(), s.moments(), s.cells_per_thread()))
        s.close()
    assert [o[2] for o in out] == [1, 2, 4]
    for o in out[1:]:
        assert np.array_equal(out[0][0], o[0])
        for c in out[0][1]:
            assert np.array_equal(out[0][1][c], o[1][c]), (o[2], c)
