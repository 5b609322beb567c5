"""All-channel launches, the mixed-precision form, and error reporting."""
import numpy as np
import pytest

from helpers import strong_diffs

pytestmark = pytest.mark.gpu


def test_batched_equals_per_channel_calls(bdmod, problems):
    p = problems(4, 20.0, 0, 20)
    a = bdmod.Context().upload(p)
    a.run_all(lanczos=True)
    b = bdmod.Context().upload(p)
    b.run_all(lanczos=True, per_channel=True)
    c = bdmod.Context().upload(p)
    for ish in range(p.ms.nsubsh):
        ra, rb = a.result(ish), b.result(ish)
        for k in ("qp", "qh", "koltun"):
            assert np.isfinite(ra[k]).all() and np.isfinite(rb[k]).all(), (ish, k)
        # a channel launched alone runs on 16-CTA clusters, batched ones on 8: the sums
        # differ in order, so members of exact degeneracies may rotate; compare what is
        # basis-independent
        for tag in ("qp", "qh"):
            assert len(ra[tag]) == len(rb[tag])
            e, z = strong_diffs(ra[tag], rb[tag])
            assert e < 1e-10 and z < 1e-10, (ish, tag, e, z)
        np.testing.assert_allclose(ra["koltun"], rb["koltun"], rtol=1e-10, atol=1e-12)
        c.sigma2_build(ish, copy=False)
        pv = p.piv
        c.lanczos_reduce(ish, pv.vec[ish], pv.n_fw[ish], pv.n_bk[ish])
        D = p.ms.no[ish]
        rc = c.dyson_solve(ish, np.diag(p.ms.orb_xe[p.ms.orb_start[ish]:p.ms.orb_start[ish] + D]))
        np.testing.assert_allclose(ra["koltun"], rc["koltun"], rtol=1e-10, atol=1e-12)
        for tag in ("qp", "qh"):
            e, z = strong_diffs(ra[tag], rc[tag])
            assert e < 1e-10 and z < 1e-10
    for x in (a, b, c):
        x.close()


def test_full_dyson_batched(bdmod, problems, golden):
    g = golden("nmax4_full")
    p = problems(4, 20.0, 0, 0)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=False)
    k = ctx.koltun_all()
    assert np.isfinite(k).all()
    for ish in range(p.ms.nsubsh):
        np.testing.assert_allclose(k[ish], g[f"c{ish}_koltun"], rtol=1e-7, atol=1e-9)
    ctx.close()


def test_mixed_precision_within_targets(bdmod, problems):
    """FP32 Lanczos vectors: every strength-carrying quasiparticle energy within 1 keV
    and every spectroscopic factor within 1e-5 of the FP64 path."""
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    ref = [ctx.result(i) for i in range(p.ms.nsubsh)]
    ctx.run_all(lanczos=True, mixed=True)
    for ish in range(p.ms.nsubsh):
        r = ctx.result(ish)
        for k in ("qp", "qh", "koltun"):
            assert np.isfinite(r[k]).all() and np.isfinite(ref[ish][k]).all(), (ish, k)
        assert (r["qp"][:, 1] > 1e-4).sum() + (r["qh"][:, 1] > 1e-4).sum() > 0
        for tag in ("qp", "qh"):
            e, z = strong_diffs(ref[ish][tag], r[tag], zmin=1e-4, etol=1e-5)
            assert e * 300.0 < 1e-3 and z < 1e-5, (ish, tag, e, z)      # |W| < 300 MeV
        # Koltun sums: the energy-weighted ones within 1 keV per unit of hole strength,
        # the strength sum within the spectroscopic-factor target
        x3 = abs(ref[ish]["koltun"][2]) + 1e-12
        dk = np.abs(r["koltun"] - ref[ish]["koltun"])
        assert dk[0] <= 1e-3 * x3 and dk[1] <= 1e-3 * x3 and dk[2] <= 1e-5 * x3, (ish, dk, x3)
    ctx.close()


def test_errors_are_status_codes(bdmod, problems):
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    with pytest.raises(bdmod.BDError) as e:
        ctx.count_poles(p.ms.nsubsh)
    assert e.value.code == bdmod.BD_ERR_ARG
    with pytest.raises(bdmod.BDError) as e:
        ctx.dyson_solve(0)                                   # no self-energy yet
    assert e.value.code == bdmod.BD_ERR_STATE
    with pytest.raises(bdmod.BDError) as e:
        ctx.result(0)                                        # no bd_run_all yet
    assert e.value.code == bdmod.BD_ERR_STATE
    fw = np.zeros((1, 2 + p.ms.no[0]))
    import ctypes as C
    n = C.c_int()
    rc = ctx.lib.bd_sigma2_build(ctx.h, 0, fw.ctypes.data_as(C.POINTER(C.c_double)), 0, C.byref(n), None, 0, None)
    assert rc == bdmod.BD_ERR_CAPACITY
    ctx.run_all(lanczos=True)                                # the context stays usable
    assert np.isfinite(ctx.koltun_all()).all()
    ctx.close()


def test_bad_interaction_lists_are_refused(bdmod, problems):
    """The device scan of the interaction list rejects an orbit out of range and a list
    that is not grouped by (charge, parity, J); the context stays usable."""
    import dataclasses
    p = problems(2, 20.0, 0, 0)
    v = p.vpp
    bad_orbit = v.iabJ.copy()
    bad_orbit[5] = ((p.ms.norb + 3) * 1024 + 0) * 128 + 1
    order = np.arange(v.n)
    order[[0, v.n - 1]] = order[[v.n - 1, 0]]                  # first and last element swapped
    ctx = bdmod.Context()
    for vv, msg in ((dataclasses.replace(v, iabJ=bad_orbit), "orbit out of range"),
                    (dataclasses.replace(v, iabJ=v.iabJ[order], icdJ=v.icdJ[order], V=v.V[order]), "not sorted")):
        with pytest.raises(bdmod.BDError) as e:
            ctx.upload(dataclasses.replace(p, vpp=vv))
        assert e.value.code == bdmod.BD_ERR_ARG and msg in str(e.value)
    ctx.upload(p)
    ctx.run_all(lanczos=False)
    assert np.isfinite(ctx.koltun_all()).all()
    ctx.close()


def test_results_all_in_one_copy(bdmod, problems):
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True)
    allr = ctx.results_all()
    for ish in range(p.ms.nsubsh):
        r = ctx.result(ish)
        for k in ("qp", "qh", "koltun"):
            assert np.array_equal(allr[ish][k], r[k]), (ish, k)
    ctx.close()


def test_non_finite_inputs_are_refused(bdmod, problems):
    """A NaN or an infinity planted (on the host) in any input gives BD_ERR_NUMERIC naming
    the input, before any kernel reads it; the context stays usable."""
    import copy
    import dataclasses
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context()
    cases = []
    v = p.vpp
    V = v.V.copy(); V[v.n // 2] = np.nan
    cases.append((dataclasses.replace(p, vpp=dataclasses.replace(v, V=V)), "matrix element"))
    V = v.V.copy(); V[-1] = np.inf
    cases.append((dataclasses.replace(p, vpp=dataclasses.replace(v, V=V)), "matrix element"))
    pr = copy.deepcopy(p.prop); pr.eh[0] = np.nan
    cases.append((dataclasses.replace(p, prop=pr), "quasihole energy"))
    pr = copy.deepcopy(p.prop); pr.fqp.reshape(-1)[3] = -np.inf
    cases.append((dataclasses.replace(p, prop=pr), "quasiparticle amplitude"))
    for bad, msg in cases:
        with pytest.raises(bdmod.BDError) as e:
            ctx.upload(bad)
        assert e.value.code == bdmod.BD_ERR_NUMERIC and msg in str(e.value), str(e.value)
    ctx.upload(p)
    piv = copy.deepcopy(p.piv)
    piv.vec[0] = piv.vec[0].copy(); piv.vec[0][0, 0] = np.nan
    with pytest.raises(bdmod.BDError) as e:
        ctx.upload_pivots(piv)
    assert e.value.code == bdmod.BD_ERR_NUMERIC and "pivots" in str(e.value)
    ctx.upload_pivots(p.piv)
    ctx.sigma2_build(0, copy=False)
    bad = p.piv.vec[0].copy(); bad[0, 0] = np.inf
    with pytest.raises(bdmod.BDError) as e:
        ctx.lanczos_reduce(0, bad, p.piv.n_fw[0], p.piv.n_bk[0])
    assert e.value.code == bdmod.BD_ERR_NUMERIC
    D = p.ms.no[0]
    s1 = np.eye(D); s1[0, 0] = np.nan
    with pytest.raises(bdmod.BDError) as e:
        ctx.dyson_solve(0, s1)
    assert e.value.code == bdmod.BD_ERR_NUMERIC
    fw, bk = ctx.sigma2_build(0)
    fw[1, 2] = np.nan
    with pytest.raises(bdmod.BDError) as e:
        ctx.dyson_rows(0, 2, fw, bk, sig1b=np.eye(D))
    assert e.value.code == bdmod.BD_ERR_NUMERIC
    ctx.run_all(lanczos=True)                                # the context stays usable
    assert np.isfinite(ctx.koltun_all()).all()
    ctx.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_graph_replay_equals_stream_launches(bdmod, problems, mixed):
    """The batched step captured in a CUDA graph and replayed gives the stream launches'
    results bit for bit, repeatedly, and its phase timings."""
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True, mixed=mixed)
    want = ctx.results_all()
    l0 = ctx.launch_count()
    for rep in range(3):
        ctx.run_all(lanczos=True, mixed=mixed, graph=True)
        got = ctx.results_all()
        for a, b in zip(want, got):
            for k in ("qp", "qh", "koltun"):
                assert np.array_equal(a[k], b[k]), (rep, k)
        t = ctx.timings()
        assert t["total"] > 0 and t["lanczos"] > 0
    assert ctx.launch_count() - l0 >= 3 * 20          # every replay counts its kernels
    ctx.set_tuning(lz_cluster=4)                      # a new tuning: captured again
    ctx.run_all(lanczos=True, mixed=mixed, graph=True)
    # four CTAs per chain sum the FP32 partials in another order: the energies move by
    # up to ~1e-7 relative, so strength is compared over the mixed form's energy window
    for a, b in zip(want, ctx.results_all()):
        for tag in ("qp", "qh"):
            e, z = strong_diffs(a[tag], b[tag], zmin=1e-4, etol=1e-5 if mixed else 1e-7)
            assert e < (1e-5 if mixed else 1e-10) and z < (1e-5 if mixed else 1e-10)
    ctx.close()


def test_autotune_picks_a_cluster_size(bdmod, problems):
    p = problems(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    lz, dy = ctx.autotune(reps=2, lanczos=True, mixed=True)
    assert lz in (4, 8, 16) and dy in (4, 8, 16)
    ctx.run_all(lanczos=True, mixed=True, graph=True)
    assert np.isfinite(ctx.koltun_all()).all()
    ctx.close()


def test_contexts_of_different_sizes_on_host_threads(bdmod, problems):
    """Two contexts with problems of different sizes driven from two host threads at
    once (kernel attributes are per process): every step gives the results the context
    gives alone, bit for bit, in both forms."""
    import threading
    probs = [problems(4, 20.0, 0, 20), problems(6, 20.0, 1, 50)]
    want = []
    for p in probs:
        c = bdmod.Context().upload(p)
        w = {}
        for mixed in (False, True):
            c.run_all(lanczos=True, mixed=mixed)
            w[mixed] = c.results_all()
        c.close()
        want.append(w)
    ctxs = [bdmod.Context().upload(p) for p in probs]
    errs = []

    def drive(j):
        try:
            for step in range(6):
                mixed = bool(step & 1)
                ctxs[j].run_all(lanczos=True, mixed=mixed, graph=(step >= 2))
                for a, b in zip(want[j][mixed], ctxs[j].results_all()):
                    for k in ("qp", "qh", "koltun"):
                        if not np.array_equal(a[k], b[k]):
                            errs.append((j, step, k))
        except Exception as ex:
            errs.append(repr(ex))
    ths = [threading.Thread(target=drive, args=(j,)) for j in range(len(ctxs))]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for c in ctxs:
        c.close()
    assert not errs, errs[:5]
