"""Pole order before the Lanczos reduction.

Reduce_SelfEn_Lncz sorts the self-energy's poles in place, forward ascending and
backward descending (source/BcDor-Self_energy_ext_Op_e.cpp:116-130), with the heap
sorts Sort_u/d_double2dim (source/BcDor-Utilities.cpp:25-94).  The unperturbed spectra
are massively degenerate (a handful of distinct energies per channel), so the order of
equal energies is the heap's, not the build order.  The rows come back in that order
(formed on the device on demand); the reduction itself visits the build order among
equal energies unless asked for the reference's (which changes only rounding).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_sorted_rows_equal_reference_program(golden, bdmod, problems):
    """Bit-exact against the rows the reference program itself left sorted in place."""
    g = golden("nmax4_lanczos20")
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    pv = p.piv
    for ish in g["keep"].tolist():
        ctx.sigma2_build(ish, copy=False)
        ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish])
        fw, bk = ctx.sigma2_sorted(ish)
        for rows, tag in ((fw, "sorted_fw"), (bk, "sorted_bk")):
            ref = g[f"c{ish}_{tag}"].reshape(rows.shape)
            assert np.array_equal(rows, ref), (ish, tag)
    ctx.close()


def _check_heap_order(ctx, orc, nsubsh):
    nties = 0
    for ish in range(nsubsh):
        fw, bk = ctx.sigma2_sorted(ish)
        fw0, bk0 = ctx.sigma2_build(ish)          # build order (the same rows the run sorted)
        for rows0, rows, desc in ((fw0, fw, False), (bk0, bk, True)):
            if not len(rows0):
                continue
            key = rows0[:, 0]
            assert np.array_equal(rows, rows0[orc.sort_perm(key, desc)]), (ish, desc)
            nties += len(key) - len(np.unique(key))
    return nties


@pytest.mark.parametrize("mixed", [False, True])
def test_heap_order_every_channel_n_max_10(bdmod, problems, oracle, mixed):
    """The bench workload (N_max=10, seed 2, 42 channels, up to 15 018 poles a channel),
    all channels in one batched run: the sorted rows are the oracle's heap sort of the
    same rows, whichever order the reduction visited."""
    p = problems(10, 16.0, 2, 100)
    orc = oracle(10, 16.0, 2, 100)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True, mixed=mixed)
    nties = _check_heap_order(ctx, orc, p.ms.nsubsh)
    assert nties > 400000            # the order of equal energies is really exercised
    ctx.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_order_of_channels_beyond_shared_memory(bdmod, problems, oracle, mixed):
    """N_max=12 (seed 3): channels of up to 28 562 poles, past the shared-memory chunk
    sort, go through the radix sort (and the heap order after it)."""
    p = problems(12, 16.0, 3, 100)
    orc = oracle(12, 16.0, 3, 100)
    ctx = bdmod.Context().upload(p)
    assert max(ctx.count_poles(i)[0] for i in range(p.ms.nsubsh)) > 16384
    ctx.run_all(lanczos=True, mixed=mixed)
    assert _check_heap_order(ctx, orc, p.ms.nsubsh) > 0
    ctx.close()


def test_reduction_visits_the_requested_order(bdmod, problems, oracle):
    """The first Lanczos vector of a chain is M p / |M p| in the order the reduction
    visits the poles: the stable order by default, the reference's heap order with
    BD_RUN_REF_ORDER (per-channel calls and the batched run alike)."""
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    pv = p.piv
    for ref in (False, True):
        for ish in (0, 1, 12):
            fw0, _ = ctx.sigma2_build(ish)
            lz = ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish], ref_order=ref)
            key = fw0[:, 0]
            order = orc.sort_perm(key, False) if ref else np.argsort(key, kind="stable")
            piv = lz["pivots"][int(np.nonzero(lz["nitr_fw"] > 0)[0][0])]
            v0 = fw0[order, 2:] @ piv
            v0 /= np.linalg.norm(v0)
            V = ctx.lanczos_vectors(ish, 0, len(lz["lz_fw"]), len(key))
            assert np.allclose(V[0], v0, atol=1e-12), (ref, ish)
    ctx.close()


def test_heap_order_per_channel_calls_and_ref_order_flag(bdmod, problems, oracle):
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    pv = p.piv
    for ish in range(p.ms.nsubsh):
        ctx.sigma2_build(ish, copy=False)
        ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish])
    assert _check_heap_order(ctx, orc, p.ms.nsubsh) > 0
    ctx.run_all(lanczos=True, ref_order=True)
    assert _check_heap_order(ctx, orc, p.ms.nsubsh) > 0
    ctx.close()


def test_sorted_rows_need_a_reduction(bdmod, problems):
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ctx.sigma2_build(0, copy=False)
    with pytest.raises(bdmod.BDError) as e:
        ctx.sigma2_sorted(0)
    assert e.value.code == bdmod.BD_ERR_STATE
    ctx.close()
