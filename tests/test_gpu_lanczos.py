"""Multi-pivot Lanczos reduction on the device."""
import numpy as np
import pytest

from helpers import first_breakdown, strong_diffs

pytestmark = pytest.mark.gpu


def test_rows_match_reference_until_breakdown(golden, bdmod, problems):
    g = golden("nmax4_lanczos20")
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    for ish in g["keep"].tolist():
        ctx.sigma2_build(ish, copy=False)
        pv = p.piv
        piv = pv.vec[ish].copy()
        lz = ctx.lanczos_reduce(ish, piv, pv.n_fw[ish], pv.n_bk[ish])
        for tag, ip in (("lz_fw", "ipiv_fw"), ("lz_bk", "ipiv_bk")):
            ref = g[f"c{ish}_{tag}"]
            got = lz[tag]
            assert got.shape == ref.shape, (ish, tag)
            nu = int(lz[ip][0])
            assert np.array_equal(lz[ip][:2 + nu], g[f"c{ish}_{ip}"][:2 + nu])
            jb = first_breakdown(ref)
            assert jb > 0
            scale = np.maximum(np.abs(ref[:jb]).max(0), 1e-300)
            err = (np.abs(got[:jb] - ref[:jb]) / scale).max()
            assert err < 1e-10, (ish, tag, jb, err)
        # side effects of the reference: pivots normalised in place
        assert np.allclose(np.linalg.norm(lz["pivots"], axis=1), 1.0)
    ctx.close()


def test_iteration_rescale_side_effect(bdmod, problems):
    """More iterations than poles: n_itr rescaled in place to int(N/sum*n + 1) and L = N
    (source/BcDor-Self_energy_ext_Op_e.cpp:216-220); ipiv records the chain starts."""
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    ish = 0
    ctx.sigma2_build(ish, copy=False)
    nfw, nbk = ctx.count_poles(ish)
    pv = p.piv
    tot = int(np.sum(pv.n_bk[ish]))
    assert tot > nbk
    lz = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish])
    expect = np.array([int(nbk / tot * v + 1.0) for v in pv.n_bk[ish]])
    assert np.array_equal(lz["nitr_bk"], expect)
    assert len(lz["lz_bk"]) == nbk
    starts = np.cumsum(expect)[:-1]
    nu = int(lz["ipiv_bk"][0])
    assert nu == len(expect) and np.array_equal(lz["ipiv_bk"][2:2 + nu - 1], starts)
    assert np.array_equal(lz["nitr_fw"], pv.n_fw[ish])          # no rescale when it fits
    ctx.close()


@pytest.mark.parametrize("mixed,tol", [(False, 1e-13), (True, 1e-5)])
def test_basis_orthonormal_and_deterministic(bdmod, problems, mixed, tol):
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    for ish in (0, 1, 12):                      # includes chains that exhaust their reachable subspace
        ctx.sigma2_build(ish, copy=False)
        pv = p.piv
        lz1 = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], mixed=mixed)
        nfw, nbk = ctx.count_poles(ish)
        for d, N, tag in ((0, nfw, "lz_fw"), (1, nbk, "lz_bk")):
            V = ctx.lanczos_vectors(ish, d, len(lz1[tag]), N, fp32=mixed)
            stored = np.abs(V).max(1) > 0          # deflated rows keep no vector
            Vs = V[stored]
            assert np.abs(Vs @ Vs.T - np.eye(len(Vs))).max() < tol, (ish, d)
            rows = lz1[tag]
            assert np.all(rows[~stored, 1:] == 0.0), (ish, d)
        lz2 = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish], mixed=mixed)
        assert np.array_equal(lz1["lz_fw"], lz2["lz_fw"]) and np.array_equal(lz1["lz_bk"], lz2["lz_bk"])
    ctx.close()


def test_rows_are_an_exact_projection(bdmod, problems):
    """The tridiagonal + fishbone layout kept by the reference equals V^T diag(E) V."""
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    for ish in (0, 12):
        fw, bk = ctx.sigma2_build(ish)
        pv = p.piv
        lz = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish])
        for d, rows_in, tag, ipk in ((0, fw, "lz_fw", "ipiv_fw"), (1, bk, "lz_bk", "ipiv_bk")):
            key = rows_in[:, 0] if d == 0 else -rows_in[:, 0]
            E = rows_in[np.argsort(key, kind="stable"), 0]
            rows = lz[tag]; L = len(rows); ipiv = lz[ipk]
            V = ctx.lanczos_vectors(ish, d, L, len(E))
            T = (V * E) @ V.T
            K = np.zeros((L, L))
            for i in range(L):
                K[i, i] = rows[i, 0]
                if i >= 1:
                    K[i, i - 1] = K[i - 1, i] = rows[i, 1]
            for nc in range(1, ipiv[0]):
                s = ipiv[nc + 1]
                if 1 <= s < L:
                    for nr in range(s, L):
                        K[s - 1, nr] = K[nr, s - 1] = rows[nr, 1 + nc]
            stored = np.abs(V).max(1) > 0
            Ts, Ks = T[np.ix_(stored, stored)], K[np.ix_(stored, stored)]
            assert np.abs(Ts - Ks).max() < 1e-10 * np.abs(E).max(), (ish, d)
            # a deflated row: no coupling to any row, a pole energy on the diagonal
            defl = ~stored
            assert np.all(K[defl][:, ~defl] == 0.0) and np.all(K[~defl][:, defl] == 0.0)
            assert np.all(np.isin(np.diag(K)[defl], E)), (ish, d)
    ctx.close()


def test_exhausted_chains_deflate(bdmod, problems, oracle):
    """The unperturbed spectra have few distinct pole energies, so every pivot's Krylov
    space is exhausted within a few steps.  The rest of each chain continues with
    eigenvectors of E that no coupling reaches (deflated rows, no stored vector), and
    the solution equals the oracle's sweep-continued chain on every strength-carrying
    solution."""
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    ndefl = 0
    for ish in (0, 12):
        ctx.sigma2_build(ish, copy=False)
        pv = p.piv
        lz = ctx.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish])
        nfw, nbk = ctx.count_poles(ish)
        V = ctx.lanczos_vectors(ish, 0, len(lz["lz_fw"]), nfw)
        ndefl += int((np.abs(V).max(1) == 0).sum())
        D = p.ms.no[ish]
        r = ctx.dyson_solve(ish, np.diag(p.ms.orb_xe[p.ms.orb_start[ish]:p.ms.orb_start[ish] + D]))
        o2 = orc.run_channel(ish, True, passes=2)
        for tag in ("qp", "qh"):
            e, z = strong_diffs(o2[tag], r[tag])
            assert e < 1e-9 and z < 1e-8, (ish, tag, e, z)
        np.testing.assert_allclose(r["koltun"], o2["koltun"], rtol=1e-9, atol=1e-9)
    assert ndefl > 0
    ctx.close()


def test_exhausted_subspace_stays_exact(bdmod, problems, oracle):
    """N_max=2 with 10 iterations per pivot: chains span their whole reachable subspace
    (the reference's rows turn NaN there).  The device continues with decoupled unit
    vectors and the reduced Dyson solution equals the un-reduced one."""
    p = problems(2, 20.0, 0, 10)
    orc = oracle(2, 20.0, 0, 10)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    k = ctx.koltun_all()
    assert np.isfinite(k).all()
    kf = np.array([orc.run_channel(i, False)["koltun"] for i in range(p.ms.nsubsh)])
    np.testing.assert_allclose(k.sum(0), kf.sum(0), rtol=1e-10)
    ko = np.array([orc.run_channel(i, True, passes=2)["koltun"] for i in range(p.ms.nsubsh)])
    np.testing.assert_allclose(k, ko, rtol=1e-9, atol=1e-9)
    ctx.close()
