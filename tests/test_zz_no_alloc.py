"""bd_lanczos_chain_noalloc, the allocation-free Lanczos entry point, against
bd_lanczos_reduce on the same channels.  Two calls in a row share the scratch
array: a long chain first, then a shorter one, then the long one again, so that
leftovers of one call would show up in the next."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _sorted_poles(rows, descending):
    """The order bd_lanczos_reduce visits by default: stable by energy, ascending (forward)
    or descending (backward)."""
    E = rows[:, 0]
    order = np.argsort(-E if descending else E, kind="stable")
    return E[order].copy(), np.ascontiguousarray(rows[order, 2:].T)


@pytest.mark.parametrize("mixed,tol", [(False, 1e-10), (True, 1e-5)])
def test_noalloc_matches_lanczos_reduce(bdmod, problems, mixed, tol):
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    dev = torch.device("cuda", 0)
    pv = p.piv
    cases = []
    for ish in (0, 12, 0):
        fw, bk = ctx.sigma2_build(ish)
        want = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], mixed=mixed)
        for d, rows, tag, ip, nit in ((0, fw, "lz_fw", "ipiv_fw", pv.n_fw[ish]),
                                      (1, bk, "lz_bk", "ipiv_bk", pv.n_bk[ish])):
            cases.append((ish, d, rows, want[tag], want[ip], nit))
    for ish, d, rows, ref, ref_ipiv, nit in cases:
        E, M = _sorted_poles(rows, descending=(d == 1))
        D = M.shape[0]
        N = len(E)
        tE = torch.from_numpy(E).to(dev)
        tM = torch.from_numpy(M).to(dev)
        cap = max(len(ref), 1)
        tout = torch.full((cap, len(pv.vec[ish]) + 1 + D), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        L, ipiv, piv, nit_out = bdmod.lanczos_chain_noalloc(tE.data_ptr(), tM.data_ptr(), N, D, pv.vec[ish], nit,
                                                            tout.data_ptr(), cap, mixed=mixed)
        got = tout.cpu().numpy()[:L]
        assert L == len(ref), (ish, d)
        assert np.array_equal(ipiv, ref_ipiv), (ish, d)
        assert np.allclose(np.linalg.norm(piv[nit_out > 0], axis=1), 1.0)
        assert np.isfinite(got).all() and np.isfinite(ref).all()
        scale = np.maximum(np.abs(ref).max(0), 1e-300)
        err = (np.abs(got - ref) / scale).max()
        assert err < tol, (ish, d, err)
    ctx.close()


def test_noalloc_rejects_chains_beyond_its_scratch(bdmod):
    """More Lanczos vectors than the scratch array holds: a clear error, nothing launched.
    The buffers are real device buffers of the sizes given, so a regression of the size
    check would show as a wrong status or wrong rows, not as a stray device access."""
    N, D, L = 40000, 1, 200
    dev = torch.device("cuda", 0)
    tE = torch.linspace(-1.0, 1.0, N, dtype=torch.float64, device=dev)
    tM = torch.ones((D, N), dtype=torch.float64, device=dev)
    tout = torch.zeros((L, 2 + D), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    with pytest.raises(bdmod.BDError) as ei:
        bdmod.lanczos_chain_noalloc(tE.data_ptr(), tM.data_ptr(), N, D, np.ones((1, 1)), np.array([L], np.int32),
                                    tout.data_ptr(), L)
    assert ei.value.code == bdmod.BD_ERR_CAPACITY and "scratch" in str(ei.value)
    assert torch.count_nonzero(tout).item() == 0
