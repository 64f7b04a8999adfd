"""Serving loop (lbmgpu_serve_run): requests admitted while others run, each
result the same alone and in the mix, against the FP64 oracle for a cavity."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U = 0.05


def _trace():
    # Reynolds numbers that keep tau >= 0.55 on these small grids (BGK at
    # tau -> 0.5 on a coarse cavity diverges, which the status word reports)
    reqs = [
        dict(kind=0, nx=16, ny=16, nz=16, reynolds=24.0, steps=120, storage="f32"),
        dict(kind=0, nx=20, ny=16, nz=12, reynolds=40.0, steps=90, storage="f32"),
        dict(kind=1, nx=48, ny=32, nz=32, reynolds=7.5, steps=60, storage="f32"),
        dict(kind=0, nx=24, ny=24, nz=24, reynolds=50.0, steps=75, storage="f16"),
        dict(kind=1, nx=40, ny=32, nz=28, reynolds=10.0, steps=50, storage="f32"),
        dict(kind=0, nx=32, ny=32, nz=32, reynolds=80.0, steps=140, storage="f32"),
    ]
    for r in reqs:
        r["arrival_s"] = 0.0
        r["keep"] = True
    return reqs


def test_serve_same_alone_and_in_mix(pkg, orc):
    reqs = _trace()
    alone = []
    for r in reqs:
        res, _ = pkg.serve_run([dict(r)], max_active=1, chunk_steps=16)
        assert res[0]["status"] == 0
        alone.append(res[0])
    mixed, upd = pkg.serve_run([dict(r) for r in reqs], max_active=6, chunk_steps=16)
    assert upd == sum(r["nx"] * r["ny"] * r["nz"] * r["steps"] for r in reqs)
    # the solves really overlapped in time
    spans = [(m["admit_s"], m["finish_s"]) for m in mixed]
    assert max(a for a, _ in spans) < min(f for _, f in spans)
    for r, a, m in zip(reqs, alone, mixed):
        assert m["status"] == 0 and m["flags"] == 0
        if r["kind"] == 0:
            # no atomics on the cavity path: identical bits
            assert np.array_equal(a["fields"], m["fields"])
        else:
            assert np.abs(a["fields"][1:] - m["fields"][1:]).max() / U < 1e-5
            assert abs(a["drag"] - m["drag"]) <= 1e-4 * abs(a["drag"])
    # the first cavity against the FP64 oracle
    r = reqs[0]
    tau = 0.5 + 3 * U * r["nx"] / r["reynolds"]
    lat = orc.cavity(r["nx"], tau, U)
    lat.step_plain(r["steps"])
    ref = orc.moments(lat)
    f = mixed[0]["fields"]
    for k, c in enumerate(("ux", "uy", "uz")):
        assert np.abs(f[1 + k] - ref[c]).max() / U < 1e-5


def test_serve_budget_and_time_limit(pkg):
    reqs = [dict(arrival_s=0.0, kind=0, nx=24, ny=24, nz=24, reynolds=36.0, steps=40, storage="f32")
            for _ in range(4)]
    # a budget that holds one solve at a time: all complete, one after another
    res, _ = pkg.serve_run(reqs, max_active=4, chunk_steps=8, hbm_budget_bytes=24 * 24 * 24 * 400 + 6e6)
    assert all(r["status"] == 0 for r in res)
    order = sorted(res, key=lambda r: r["admit_s"])
    for a, b in zip(order, order[1:]):
        assert b["admit_s"] >= a["finish_s"] - 1e-6
    # a time limit cuts long requests off cleanly
    long = [dict(arrival_s=0.0, kind=0, nx=32, ny=32, nz=32, reynolds=48.0, steps=10 ** 7, storage="f32")]
    res, _ = pkg.serve_run(long, max_active=1, chunk_steps=100, time_limit_s=0.5)
    assert res[0]["status"] == 6  # LBM_ERR_STATE: stopped by the time limit
