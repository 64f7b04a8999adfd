"""lbmgpu_batch_step_noalloc: the batched-cavity step for callers that cannot
allocate device memory (they own the population buffers; the library's
working data lives in a fixed device array).  Two calls in a row must give
what the allocating entry point (lbmgpu_batch_*) gives, in every storage
type, with the newest state in pop_a after an even step count and in pop_b
after an odd one.  Kept in its own file so that a run stopping at the first
failure has already run every other test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# Both sides store the same post-collision values; the comparison takes the
# moments of the stored populations against the allocating path's moments of
# the same state one step earlier, which an unforced BGK collision conserves
# up to the rounding of the stored values: |f - w| <= ~0.02 on these lids, so
# one link is rounded by up to 1e-5 (FP16, 2^-11) or 8e-5 (BF16, 2^-8), and
# 19 of them give the bounds below (FP32: the FP32 collision's own rounding).
TOL = {"f32": (1e-6, 4e-6), "f16": (2e-4, 2e-3), "bf16": (2e-3, 2e-2)}  # rho, |u| / lid
DTYPE = {"f32": "float32", "f16": "float16", "bf16": "bfloat16"}


def _moments_from_pops(pops, base, S, dims):
    """rho, ux, uy, uz of every cavity from shifted populations (f - w)."""
    import oracle

    out = []
    for p, (nx, ny, nz) in enumerate(dims):
        N = nx * ny * nz
        f = np.stack([pops[base[p] + l * S[p]: base[p] + l * S[p] + N] for l in range(19)]).astype(np.float64)
        rho = 1.0 + f.sum(axis=0)
        u = [np.tensordot(c, f, axes=(0, 0)) / rho for c in (oracle.CX19, oracle.CY19, oracle.CZ19)]
        out.append([a.reshape(nz, ny, nx) for a in (rho, *u)])
    return out


@pytest.mark.parametrize("storage", ["f32", "f16", "bf16"])
def test_noalloc_matches_batch_two_calls(pkg, storage):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    dims = rng.integers(8, 24, size=(5, 3))
    taus = rng.uniform(0.55, 0.9, size=5)
    base, S, total = pkg.batch_layout(dims, storage)
    dt = getattr(torch, DTYPE[storage])
    a = torch.zeros(total, dtype=dt, device="cuda")  # f - w = 0: rest state
    b = torch.zeros(total, dtype=dt, device="cuda")
    torch.cuda.synchronize()
    ref = pkg.Batch(dims, taus, lid=0.05, storage=storage)
    ref.init()
    tr, tu = TOL[storage]
    dl = [tuple(int(v) for v in d) for d in dims]
    # The buffers hold post-collision populations of the last step; an
    # unforced BGK collision keeps rho and rho u, so their moments are the
    # pre-collision moments of that step, which the allocating entry point
    # reports after one step fewer (its read-back streams the stored state).
    # The second call runs an odd count: its newest state is in pop_b.
    for call, first, nsteps, ref_steps, newest in ((1, 1, 40, 39, a), (2, 0, 41, 41, b)):
        st = pkg.batch_step_noalloc(dims, taus, 0.05, storage, a.data_ptr(), b.data_ptr(), first, nsteps)
        assert (st == 0).all()
        ref.step(ref_steps)
        got = _moments_from_pops(newest.float().cpu().numpy(), base, S, dl)
        for p in range(len(taus)):
            m = ref.moments(p)
            for k, c in enumerate(("rho", "ux", "uy", "uz")):
                tol = tr if c == "rho" else tu * 0.05
                assert np.abs(got[p][k] - m[c]).max() < tol, (storage, call, p, c)


def test_noalloc_refuses_stream_capture(pkg):
    """Each call copies its tables from host memory, so it cannot be captured:
    on a capturing stream it returns LBM_ERR_STATE and enqueues nothing."""
    torch = pytest.importorskip("torch")
    dims = [(8, 8, 8)]
    _, _, total = pkg.batch_layout(dims, "f32")
    a = torch.zeros(total, dtype=torch.float32, device="cuda")
    b = torch.zeros(total, dtype=torch.float32, device="cuda")
    pkg.batch_step_noalloc(dims, [0.8], 0.05, "f32", a.data_ptr(), b.data_ptr(), 1, 2)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.graph(g, stream=s):
        try:
            pkg.batch_step_noalloc(dims, [0.8], 0.05, "f32", a.data_ptr(), b.data_ptr(), 0, 2, stream=s.cuda_stream)
        except pkg.LbmError as e:
            err = e
        a.mul_(1.0)  # the graph has one node of its own
    assert err is not None and err.status == 6, err
    g.replay()
    torch.cuda.synchronize()


def test_noalloc_rejects_oversized_batch(pkg):
    dims = np.full((1025, 3), 4)
    with pytest.raises(pkg.LbmError) as e:
        pkg.batch_step_noalloc(dims, np.full(1025, 0.8), 0.05, "f32", 1, 1, 1, 1)
    assert e.value.status == 1 and "1024" in str(e.value)
