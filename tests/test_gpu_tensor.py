"""The mixed form's coupling build on the tensor cores (k_coupling_tc.cu) against the
FP64 build (k_poles) on dressed propagators: the same energies bit for bit, couplings
within the TF32 three-product bound, and the chain's solutions on top of each."""
import numpy as np
import pytest

from helpers import koltun_energy, strong_diffs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nmax,hw,seed,nit", [(4, 20.0, 0, 20), (6, 20.0, 1, 50)])
def test_tensor_core_couplings_match_fp64(bdmod, problems, nmax, hw, seed, nit):
    p = problems(nmax, hw, seed, nit)
    ns = p.ms.nsubsh
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    assert not ctx.tensor_couplings()                 # FP64 form: the FP64 build
    ctx.run_all(lanczos=True, mixed=True)
    assert not ctx.tensor_couplings()                 # one-hot amplitudes: the FP64 build
    ctx.dressed_propagator(1e-3, 2)                   # a dressed propagator
    ctx.run_all(lanczos=True, mixed=True)
    assert ctx.tensor_couplings()
    tc = [ctx.sigma2_sorted(i) for i in range(ns)]
    res_tc = ctx.results_all()
    ctx.run_all(lanczos=True, mixed=True, fp64_couplings=True)
    assert not ctx.tensor_couplings()
    ref = [ctx.sigma2_sorted(i) for i in range(ns)]
    res_ref = ctx.results_all()
    worst = 0.0
    for ish in range(ns):
        for got, want in zip(tc[ish], ref[ish]):
            assert got.shape == want.shape
            if not len(want):
                continue
            assert np.array_equal(got[:, 0], want[:, 0]), ish   # energies: k_poles's operations
            scale = np.abs(want[:, 2:]).max()
            if scale == 0.0:
                assert np.abs(got[:, 2:]).max() == 0.0
                continue
            err = np.abs(got[:, 2:] - want[:, 2:]).max() / scale
            worst = max(worst, err)
            # S2 = sum_d M^2 of every pole, from the same couplings
            np.testing.assert_allclose(got[:, 1], want[:, 1], rtol=1e-4, atol=1e-6 * scale * scale)
    assert worst < 1e-5, worst
    # the chain on either build: strength-carrying solutions within 1 keV (the mixed form's
    # target; dense dressed spectra move interior solutions for perturbations of M this
    # small) and the Koltun energy
    for a, b in zip(res_ref, res_tc):
        for tag in ("qp", "qh"):
            ra, rb = a[tag], b[tag]
            for r in ra[ra[:, 1] > 1e-2]:
                dw = np.abs(rb[:, 0] - r[0]).min()
                assert dw < 1e-3, (tag, r[0], dw)
            _, z = strong_diffs(ra, rb, zmin=1e-2, etol=1e-5)
            assert z < 1e-4, (tag, z)
    ka, kb = koltun_energy([r["koltun"] for r in res_ref]), koltun_energy([r["koltun"] for r in res_tc])
    assert abs(ka - kb) <= 1e-5 * abs(ka)
    ctx.close()


def test_tensor_core_couplings_in_graph_replay(bdmod, problems):
    """The tensor-core build captured in the step's graph gives the stream launches'
    results bit for bit."""
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    ctx.dressed_propagator(1e-3, 2)
    ctx.run_all(lanczos=True, mixed=True)
    want = ctx.results_all()
    for _ in range(2):
        ctx.run_all(lanczos=True, mixed=True, graph=True)
        assert ctx.tensor_couplings()
        for a, b in zip(want, ctx.results_all()):
            for k in ("qp", "qh", "koltun"):
                assert np.array_equal(a[k], b[k]), k
    ctx.close()
