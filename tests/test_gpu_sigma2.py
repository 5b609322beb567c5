"""Sigma(2) build and static self-energy on the device: bit-exact against the reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sigma2_and_ehf_bitexact_vs_reference(golden, bdmod, problems):
    g = golden("nmax4_full")
    p = problems(4, 20.0, 0, 0)
    ctx = bdmod.Context().upload(p)
    keep = set(g["keep"].tolist())
    for ish in range(p.ms.nsubsh):
        fw, bk = ctx.sigma2_build(ish)
        for tag, a in (("sig_fw", fw), ("sig_bk", bk)):
            chk = np.array([len(a), a.sum(), (a * a).sum(), np.abs(a).max() if len(a) else 0.0])
            assert np.array_equal(chk, g[f"c{ish}_{tag}_sum"]), (ish, tag)
            if ish in keep:
                assert np.array_equal(a, g[f"c{ish}_{tag}"]), (ish, tag)
        assert np.array_equal(ctx.ehf(ish), g[f"c{ish}_sig_hf"]), ish
    ctx.close()


def test_sigma2_bitexact_vs_oracle_nmax6(bdmod, problems, oracle):
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    for ish in range(p.ms.nsubsh):
        assert ctx.count_poles(ish) == orc.count_poles(ish)
        fw, bk = ctx.sigma2_build(ish)
        ofw, obk = orc.sigma2(ish)
        assert np.array_equal(fw, ofw) and np.array_equal(bk, obk), ish
        assert np.array_equal(ctx.ehf(ish), orc.ehf(ish)), ish
    ctx.close()


def test_dressed_propagator_sigma2(bdmod, synth, oracle_mod):
    """Non one-hot amplitudes (several fragments per orbit) exercise the full V' X f
    contraction; the device keeps the reference's operation order, so rows stay bit-exact."""
    p = synth.make_problem(2, 20.0, 5, 5)
    rng = np.random.default_rng(11)
    pr = p.prop
    # rotate each subshell's particle amplitudes by a random orthogonal matrix
    for s in range(p.ms.nsubsh):
        n, st, D = pr.np_[s], pr.p_start[s], p.ms.no[s]
        if n > 1:
            q, _ = np.linalg.qr(rng.standard_normal((n, n)))
            pr.fqp[st:st + n, :D] = q @ pr.fqp[st:st + n, :D]
            pr.ep[st:st + n] += rng.uniform(-1, 1, n)
    orc = oracle_mod.Oracle().bind(p)
    ctx = bdmod.Context().upload(p)
    for ish in range(p.ms.nsubsh):
        fw, bk = ctx.sigma2_build(ish)
        ofw, obk = orc.sigma2(ish)
        assert np.array_equal(fw, ofw) and np.array_equal(bk, obk), ish
    ctx.close()
