"""lbmgpu_batch_step_noalloc: the batched-cavity step for callers that cannot
allocate device memory (they own the population buffers; the library's
working data lives in a fixed device array).  Two calls in a row must give
what the allocating entry point (lbmgpu_batch_*) gives.  Kept in its own file
so that a run stopping at the first failure has already run every other test."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_batch_two_calls(pkg):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    dims = rng.integers(8, 24, size=(5, 3))
    taus = rng.uniform(0.55, 0.9, size=5)
    base, S, total = pkg.batch_layout(dims, "f32")
    a = torch.zeros(total, dtype=torch.float32, device="cuda")  # f - w = 0: rest state
    b = torch.zeros(total, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    ref = pkg.Batch(dims, taus, lid=0.05, storage="f32")
    ref.init()
    # The buffers hold post-collision populations of the last step; an
    # unforced BGK collision keeps rho and rho u, so their moments are the
    # pre-collision moments of that step, which the allocating entry point
    # reports after one step fewer (its read-back streams the stored state).
    for call, first, ref_steps in ((1, 1, 39), (2, 0, 40)):
        st = pkg.batch_step_noalloc(dims, taus, 0.05, "f32", a.data_ptr(), b.data_ptr(), first, 40)
        assert (st == 0).all()
        ref.step(ref_steps)
        got = _moments_from_pops(a.cpu().numpy(), base, S, [tuple(int(v) for v in d) for d in dims])
        for p in range(len(taus)):
            m = ref.moments(p)
            for k, c in enumerate(("rho", "ux", "uy", "uz")):
                tol = 1e-6 if c == "rho" else 4e-6 * 0.05
                assert np.abs(got[p][k] - m[c]).max() < tol, (call, p, c)


def test_noalloc_rejects_oversized_batch(pkg):
    dims = np.full((1025, 3), 4)
    with pytest.raises(pkg.LbmError) as e:
        pkg.batch_step_noalloc(dims, np.full(1025, 0.8), 0.05, "f32", 1, 1, 1, 1)
    assert e.value.status == 1 and "1024" in str(e.value)
