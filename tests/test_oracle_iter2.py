"""Second iteration with a dressed propagator: the oracle against the reference program
run on the same truncated propagator (tests/golden/*_iter2.npz)."""
import dataclasses

import numpy as np
import pytest

from helpers import strong_diffs


def _iter2_problem(synth, golden, problems, name):
    g = golden(name)
    nmax, hw, seed, nit = (int(g["meta"][0]), float(g["meta"][1]), int(g["meta"][2]), int(g["meta"][3]))
    p1 = problems(nmax, hw, seed, nit)
    nspb = p1.prop.nspb
    prop2 = synth.propagator_from_arrays(nspb, g["p_np"], g["p_nh"], g["p_ep"], g["p_eh"], g["p_fqp"], g["p_fqh"])
    return g, p1, dataclasses.replace(p1, prop=prop2), nit


@pytest.mark.parametrize("name", ["nmax2_full_iter2", "nmax4_lanczos20_iter2"])
def test_dressed_sigma2_and_ehf_bit_exact(synth, oracle_mod, golden, problems, name):
    g, _, p2, _ = _iter2_problem(synth, golden, problems, name)
    orc = oracle_mod.Oracle().bind(p2)
    for ish in range(p2.ms.nsubsh):
        fw, bk = orc.sigma2(ish)
        for tag, a in (("sig_fw", fw), ("sig_bk", bk)):
            ref = g[f"c{ish}_{tag}_sum"]
            got = np.array([len(a), a.sum(), (a * a).sum(), np.abs(a).max() if len(a) else 0.0])
            assert np.array_equal(got, ref), (ish, tag, got, ref)
        assert np.array_equal(orc.ehf(ish), g[f"c{ish}_sig_hf"]), ish


def test_dressed_full_dyson_matches_reference(synth, oracle_mod, golden, problems):
    g, _, p2, _ = _iter2_problem(synth, golden, problems, "nmax2_full_iter2")
    orc = oracle_mod.Oracle().bind(p2)
    for ish in (1, 2, 3, 4):           # the smaller channels keep the CPU suite short
        r = orc.run_channel(ish, False)
        for tag in ("qp", "qh"):
            assert len(r[tag]) == int(g[f"c{ish}_{tag}_n"][0])
            e, z = strong_diffs(g[f"c{ish}_{tag}_strong"], r[tag])
            assert e < 1e-8 and z < 1e-8, (ish, tag, e, z)
        np.testing.assert_allclose(r["koltun"], g[f"c{ish}_koltun"], rtol=1e-7, atol=1e-9)


def test_dressed_lanczos_rows_match_reference(synth, oracle_mod, golden, problems):
    g, _, p2, _ = _iter2_problem(synth, golden, problems, "nmax4_lanczos20_iter2")
    orc = oracle_mod.Oracle().bind(p2)
    for ish in g["keep"].tolist():
        fw, bk = orc.sigma2(ish)
        pv = p2.piv
        lz = orc.reduce_lanczos(ish, fw, bk, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], 1)
        for tag in ("lz_fw", "lz_bk"):
            np.testing.assert_array_equal(lz[tag], g[f"c{ish}_{tag}"])


def test_update_rule_reproduces_fixture_propagator(synth, oracle_mod, golden, problems):
    """The oracle's first iteration (the reference's algorithm: full Dyson through LAPACK)
    turned into the next propagator gives the fixture's propagator."""
    g, p1, _, _ = _iter2_problem(synth, golden, problems, "nmax2_full_iter2")
    orc = oracle_mod.Oracle().bind(p1)
    res = [orc.run_channel(i, False) for i in range(p1.ms.nsubsh)]
    z_cut, max_frag = float(g["trunc"][0]), int(g["trunc"][1])
    dp = oracle_mod.dressed_propagator(p1.ms, res, p1.prop.nspb, z_cut, max_frag)
    assert np.array_equal(dp["np"], g["p_np"]) and np.array_equal(dp["nh"], g["p_nh"])
    np.testing.assert_allclose(dp["ep"], g["p_ep"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(dp["eh"], g["p_eh"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(np.abs(dp["fqp"]).reshape(-1), np.abs(g["p_fqp"]).reshape(-1), atol=1e-10)
    np.testing.assert_allclose(np.abs(dp["fqh"]).reshape(-1), np.abs(g["p_fqh"]).reshape(-1), atol=1e-10)
    d = oracle_mod.quick_n_dirty_diff(p1.prop.ep, p1.prop.eh, dp["ep"], dp["eh"])
    assert d == pytest.approx(float(g["diff1"][0]), rel=1e-12)
