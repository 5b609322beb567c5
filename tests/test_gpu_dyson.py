"""Dyson eigensolve on the device."""
import numpy as np
import pytest

from helpers import koltun_energy, strong_diffs

pytestmark = pytest.mark.gpu


def test_full_dyson_matches_reference(golden, bdmod, problems):
    """Plain Sigma(2) + full Dyson diagonalisation (N_max=4, hw=20, seed 0): every
    strength-carrying solution within 1e-8 relative in energy, Koltun within 1e-7."""
    g = golden("nmax4_full")
    p = problems(4, 20.0, 0, 0)
    ctx = bdmod.Context().upload(p)
    for ish in range(p.ms.nsubsh):
        ctx.sigma2_build(ish, copy=False)
        D = p.ms.no[ish]
        s1b = np.diag(p.ms.orb_xe[p.ms.orb_start[ish]:p.ms.orb_start[ish] + D])
        r = ctx.dyson_solve(ish, s1b)
        for tag in ("qp", "qh"):
            assert len(r[tag]) == int(g[f"c{ish}_{tag}_n"][0]), (ish, tag)
            e, z = strong_diffs(g[f"c{ish}_{tag}_strong"], r[tag])
            assert e < 1e-8 and z < 1e-8, (ish, tag, e, z)
            assert np.all(np.diff(r[tag][:, 0]) <= 0)          # descending W
        np.testing.assert_allclose(r["koltun"], g[f"c{ish}_koltun"], rtol=1e-7, atol=1e-9)
    ctx.close()


def test_lanczos_dyson_equals_unreduced_solution(bdmod, problems, oracle):
    """Lanczos 50 it/pivot at N_max=6: the reduced Dyson solutions equal the oracle's
    (two-sweep) ones and the un-reduced Dyson solution of the same Sigma(2)."""
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    Kg = np.zeros(3); Kf = np.zeros(3)
    for ish in range(p.ms.nsubsh):
        o2 = orc.run_channel(ish, True, passes=2)
        ctx.sigma2_build(ish, copy=False)
        pv = p.piv
        ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish])
        r = ctx.dyson_solve(ish, o2["sig_1b"])
        for tag in ("qp", "qh"):
            assert len(r[tag]) == len(o2[tag])
            e, z = strong_diffs(o2[tag], r[tag])
            assert e < 1e-9 and z < 1e-8, (ish, tag, e, z)
        np.testing.assert_allclose(r["koltun"], o2["koltun"], rtol=1e-9, atol=1e-9)
        fw, bk = orc.sigma2(ish)
        Kf += orc.dyson(ish, o2["sig_1b"], o2["sig_hf"], 2, fw, bk)["koltun"]
        Kg += r["koltun"]
    assert abs(koltun_energy(Kg) - koltun_energy(Kf)) < 1e-9 * abs(koltun_energy(Kf))
    ctx.close()


def test_dyson_on_supplied_rows(bdmod, problems, oracle):
    """bd_dyson_rows: Dyson on caller-supplied self-energy rows (Lanczos rows of the
    oracle, and plain Sigma(2) rows)."""
    p = problems(4, 20.0, 0, 20)
    orc = oracle(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    for ish in (0, 3, 9):
        o2 = orc.run_channel(ish, True, passes=2)
        r = ctx.dyson_rows(ish, o2["NDEN"], o2["lz_fw"], o2["lz_bk"], o2["ipiv_fw"], o2["ipiv_bk"],
                           o2["sig_1b"], o2["sig_hf"])
        for tag in ("qp", "qh"):
            e, z = strong_diffs(o2[tag], r[tag])
            assert e < 1e-10 and z < 1e-9, (ish, tag, e, z)
        np.testing.assert_allclose(r["koltun"], o2["koltun"], rtol=1e-10, atol=1e-10)
        fw, bk = orc.sigma2(ish)
        full = orc.dyson(ish, o2["sig_1b"], o2["sig_hf"], 2, fw, bk)
        r2 = ctx.dyson_rows(ish, 2, fw, bk, None, None, o2["sig_1b"], o2["sig_hf"])
        np.testing.assert_allclose(r2["koltun"], full["koltun"], rtol=1e-10, atol=1e-10)
    ctx.close()


def test_sum_rules(bdmod, problems):
    """Every channel's spectroscopic factors add up to D (completeness of the D
    one-body components), and the Koltun occupation is finite and near A=16."""
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    A = 0.0
    for ish in range(p.ms.nsubsh):
        r = ctx.result(ish)
        z = r["qp"][:, 1].sum() + r["qh"][:, 1].sum()
        assert abs(z - p.ms.no[ish]) < 1e-9, (ish, z)
        A += r["koltun"][2]
    assert 15.0 < A < 17.5
    ctx.close()
