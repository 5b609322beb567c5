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


def test_dressed_orders_near_1000_against_lapack(bdmod, problems, oracle):
    """The eigensolver where the dressed spectra put it: N_max=10 second iteration (Z >= 1e-3,
    two fragments per side), whose chains build every vector, so the Dyson matrices keep
    orders near 1 000 (Householder in FP64 on a cluster, Sturm bisection in double-float,
    inverse iteration in FP64).  The same Lanczos rows go to bd_dyson_rows and to the
    oracle's DysonMatrix with LAPACK dsyevd: every solution with Z > 1e-6 within 1e-8
    relative in energy and 1e-8 in Z, Koltun sums within 1e-7 relative."""
    p = problems(10, 16.0, 2, 100)
    orc = oracle(10, 16.0, 2, 100)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    ctx.dressed_propagator(1e-3, 2)
    pv = p.piv
    orders = []
    for ish in (0, 21, 9):
        ctx.sigma2_build(ish, copy=False)
        lz = ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish])
        D = int(p.ms.no[ish])
        n = D + len(lz["lz_fw"]) + len(lz["lz_bk"])
        orders.append(n)
        s1 = np.diag(p.ms.orb_xe[p.ms.orb_start[ish]:p.ms.orb_start[ish] + D])
        sh = ctx.ehf(ish)
        ef = orc.efermi(ish)
        got = ctx.dyson_rows(ish, lz["NDEN"], lz["lz_fw"], lz["lz_bk"], lz["ipiv_fw"], lz["ipiv_bk"], sig1b=s1,
                             sighf=sh, efermi=ef)
        ref = orc.dyson(ish, s1, sh, lz["NDEN"], lz["lz_fw"], lz["lz_bk"], lz["n_piv_fw"], lz["ipiv_fw"],
                        lz["n_piv_bk"], lz["ipiv_bk"])
        for tag in ("qp", "qh"):
            assert len(got[tag]) == len(ref[tag]), (ish, tag)
            e, z = strong_diffs(ref[tag], got[tag])
            assert e < 1e-8 and z < 1e-8, (ish, tag, n, e, z)
        np.testing.assert_allclose(got["koltun"], ref["koltun"], rtol=1e-7, atol=1e-9)
    assert max(orders) > 800, orders
    ctx.close()


def test_dyson_rows_beyond_eight_thousand_deflated_poles(bdmod, problems, oracle):
    """Plain Sigma(2) rows of one channel with 9 000 uncoupled poles appended (every M
    zero, distinct energies above the forward and below the backward poles): the
    uncoupled poles deflate, so the compact eigenproblem is the oracle's, while the
    placement ranks more than 8 192 rows (k_place's several row groups) and the Koltun
    sums run over more than 256 quasiholes (k_koltun's eight CTAs).  Every appended pole
    comes back once as [E, 0, 0 ..], both lists descend, the rest and the Koltun sums
    are the oracle's."""
    p = problems(4, 20.0, 0, 20)
    orc = oracle(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ish = 0
    o2 = orc.run_channel(ish, True, passes=2)
    fw, bk = orc.sigma2(ish)
    full = orc.dyson(ish, o2["sig_1b"], o2["sig_hf"], 2, fw, bk)
    D = fw.shape[1] - 2
    rng = np.random.default_rng(7)
    nfx, nbx = 4000, 5000
    efx = fw[:, 0].max() + 1.0 + np.sort(rng.uniform(0.0, 300.0, nfx))
    ebx = bk[:, 0].min() - 1.0 - np.sort(rng.uniform(0.0, 300.0, nbx))
    assert len(np.unique(efx)) == nfx and len(np.unique(ebx)) == nbx
    fwx = np.zeros((nfx, 2 + D)); fwx[:, 0] = efx
    bkx = np.zeros((nbx, 2 + D)); bkx[:, 0] = ebx
    big_fw, big_bk = np.vstack([fw, fwx[::-1]]), np.vstack([bk, bkx[rng.permutation(nbx)]])
    assert D + len(big_fw) + len(big_bk) > 8192
    r = ctx.dyson_rows(ish, 2, big_fw, big_bk, None, None, o2["sig_1b"], o2["sig_hf"])
    assert len(r["qp"]) == len(full["qp"]) + nfx and len(r["qh"]) == len(full["qh"]) + nbx
    assert len(r["qh"]) > 256
    for tag, extra in (("qp", efx), ("qh", ebx)):
        got = r[tag]
        assert np.all(np.diff(got[:, 0]) <= 0), tag            # descending W
        hit = np.isin(got[:, 0], extra)
        assert hit.sum() == len(extra), tag                     # each appended pole once
        assert np.all(got[hit, 1:] == 0.0), tag                 # with Z = 0 and x = 0
        e, z = strong_diffs(full[tag], got[~hit])
        assert e < 1e-10 and z < 1e-9, (tag, e, z)
    np.testing.assert_allclose(r["koltun"], full["koltun"], rtol=1e-10, atol=1e-10)
    ctx.close()


def test_dyson_rows_beyond_the_cluster_layout_report_capacity(bdmod, problems, oracle):
    """A deflated Dyson matrix larger than the cluster reduction's shared-memory layout
    (the channel's plain Sigma(2) rows thirty times over, energies spread apart, so
    about 9 000 coupled poles): BD_ERR_CAPACITY with a message, and the context then
    solves the channel's own rows as the oracle does."""
    p = problems(4, 20.0, 0, 20)
    orc = oracle(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ish = 0
    o2 = orc.run_channel(ish, True, passes=2)
    fw, bk = orc.sigma2(ish)
    reps = []
    for q in range(30):
        r = fw.copy()
        r[:, 0] += 1e-3 * q
        reps.append(r)
    big_fw = np.vstack(reps)
    with pytest.raises(bdmod.BDError) as ei:
        ctx.dyson_rows(ish, 2, big_fw, bk, None, None, o2["sig_1b"], o2["sig_hf"])
    assert ei.value.code == bdmod.BD_ERR_CAPACITY and "shared memory" in str(ei.value)
    full = orc.dyson(ish, o2["sig_1b"], o2["sig_hf"], 2, fw, bk)
    r2 = ctx.dyson_rows(ish, 2, fw, bk, None, None, o2["sig_1b"], o2["sig_hf"])
    for tag in ("qp", "qh"):
        e, z = strong_diffs(full[tag], r2[tag])
        assert e < 1e-10 and z < 1e-9, (tag, e, z)
    np.testing.assert_allclose(r2["koltun"], full["koltun"], rtol=1e-10, atol=1e-10)
    ctx.close()
