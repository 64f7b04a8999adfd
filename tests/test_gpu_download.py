"""Asynchronous moment read-back (lbmgpu_download_all_f32_async): the host
buffer holds exactly what the synchronous read-back returns for the same
state, also when the next steps are already enqueued behind the copy."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solver(pkg):
    s = pkg.Solver(pkg.channel_config(48, 24, 20, 0.6, u_in=0.05, storage="f16", graph_steps=8))
    s.init()
    return s


def test_async_download_equals_sync_and_pipelines(pkg):
    L = pkg.load()
    a, b = _solver(pkg), _solver(pkg)
    n = 4 * a.ncell
    bufs = []
    for _ in range(2):
        p = C.c_void_p()
        pkg.check(L.lbmgpu_host_alloc(n * 4, C.byref(p)))
        bufs.append(p)
    try:
        # a: two asynchronous read-backs with 16 steps enqueued between them
        a.step(16)
        pkg.check(L.lbmgpu_download_all_f32_async(a.h, bufs[0]))
        a.step(16)
        pkg.check(L.lbmgpu_download_all_f32_async(a.h, bufs[1]))
        pkg.check(L.lbmgpu_download_wait(a.h))
        got = [np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_float)), shape=(n,)).copy() for p in bufs]
        # b: the same steps, synchronous read-backs
        ref = []
        for _ in range(2):
            b.step(16)
            out = np.empty(n, np.float32)
            pkg.check(L.lbmgpu_download_all_f32(b.h, out.ctypes.data_as(C.c_void_p)))
            ref.append(out)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
        assert not np.array_equal(got[0], got[1])
    finally:
        for p in bufs:
            L.lbmgpu_host_free(p)
        a.close()
        b.close()


@pytest.mark.parametrize("memory", ["pageable", "pinned"])
def test_update_markers_keeps_graphs_and_moves_the_body(pkg, orc, memory):
    """lbmgpu_update_markers: the same positions change nothing (graphs kept);
    shifted positions before the first step give the run of a body
    registered there; from pageable memory and from pinned memory
    (lbmgpu_host_alloc)."""
    L = pkg.load()
    n, D, c = 200, 8.0, (20.0, 12.0, 10.0)
    mk = orc.fibonacci_sphere(n, D, c)
    bufs = []

    def host(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if memory == "pageable":
            return a
        p = C.c_void_p()
        pkg.check(L.lbmgpu_host_alloc(a.nbytes, C.byref(p)))
        bufs.append(p)
        h = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_double)), shape=a.shape)
        h[...] = a
        return h

    xyz = host(np.stack([mk["x"], mk["y"], mk["z"]]))
    ds = host(mk["ds"])

    def solver(pos):
        s = pkg.Solver(pkg.channel_config(48, 24, 20, 0.6, u_in=0.05, graph_steps=4))
        s.init()
        s.set_markers(pos, ds, D / 2.0, c, m_max=3)
        return s

    dp = C.POINTER(C.c_double)
    a, b = solver(xyz), solver(xyz)
    for _ in range(3):
        a.step(8)
        pkg.check(L.lbmgpu_update_markers(b.h, xyz.ctypes.data_as(dp), ds.ctypes.data_as(dp)))
        b.step(8)
    assert np.abs(a.moments()["ux"] - b.moments()["ux"]).max() < 1e-6
    fa, fb = a.forces(), b.forces()
    assert np.array_equal(fa[:, 7], fb[:, 7]) and np.abs(fa[:, :3] - fb[:, :3]).max() < 1e-5 * np.abs(fa[:, :3]).max()
    # a small move that keeps every stencil inside the band set up for xyz
    shifted = host(xyz + np.array([[0.1], [0.0], [0.0]]))
    d, e = solver(shifted), solver(xyz)
    pkg.check(L.lbmgpu_update_markers(e.h, shifted.ctypes.data_as(dp), ds.ctypes.data_as(dp)))
    d.step(16)
    e.step(16)
    assert e.status() == 0
    fd, fe = d.forces(), e.forces()
    assert np.abs(fd[:, :3] - fe[:, :3]).max() < 1e-5 * np.abs(fd[:, :3]).max()
    for x in (a, b, d, e):
        x.close()
    for p in bufs:
        L.lbmgpu_host_free(p)
    with pytest.raises(pkg.LbmError):
        s = pkg.Solver(pkg.channel_config(16, 8, 8, 0.6))
        s.init()
        pkg.check(L.lbmgpu_update_markers(s.h, xyz.ctypes.data_as(dp), ds.ctypes.data_as(dp)))
