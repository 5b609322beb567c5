"""Pole order before the Lanczos reduction.

Reduce_SelfEn_Lncz sorts the self-energy's poles in place, forward ascending and
backward descending (source/BcDor-Self_energy_ext_Op_e.cpp:116-130), with the heap
sorts Sort_u/d_double2dim (source/BcDor-Utilities.cpp:25-94).  The unperturbed spectra
are massively degenerate (a handful of distinct energies per channel), so the order of
equal energies is the heap's, not the build order.  The FP64 path reproduces it; the
FP32 form keeps the build order among equal energies.
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


def _check_heap_order(ctx, orc, nsubsh, mixed):
    nties = 0
    for ish in range(nsubsh):
        fw, bk = ctx.sigma2_sorted(ish)
        fw0, bk0 = ctx.sigma2_build(ish)          # build order (the same rows the run sorted)
        for rows0, rows, desc in ((fw0, fw, False), (bk0, bk, True)):
            if not len(rows0):
                continue
            key = rows0[:, 0]
            if mixed:
                perm = np.argsort(-key if desc else key, kind="stable")
            else:
                perm = orc.sort_perm(key, desc)
            assert np.array_equal(rows, rows0[perm]), (ish, desc)
            nties += len(key) - len(np.unique(key))
    return nties


@pytest.mark.parametrize("mixed", [False, True])
def test_heap_order_every_channel_n_max_10(bdmod, problems, oracle, mixed):
    """The bench workload (N_max=10, seed 2, 42 channels, up to 15 018 poles a channel),
    all channels in one batched run: the FP64 path's order is the oracle's heap sort of
    the same rows, the FP32 form's the stable sort."""
    p = problems(10, 16.0, 2, 100)
    orc = oracle(10, 16.0, 2, 100)
    ctx = bdmod.Context().upload(p)
    ctx.run_all(lanczos=True, mixed=mixed)
    nties = _check_heap_order(ctx, orc, p.ms.nsubsh, mixed)
    assert nties > 400000            # the order of equal energies is really exercised
    ctx.close()


@pytest.mark.parametrize("mixed", [False, True])
def test_order_of_channels_beyond_shared_memory(bdmod, problems, oracle, mixed):
    """N_max=12 (seed 3): channels of up to 28 562 poles, past the shared-memory chunk
    sort, go through the radix sort (and, in FP64, the heap order after it)."""
    p = problems(12, 16.0, 3, 100)
    orc = oracle(12, 16.0, 3, 100)
    ctx = bdmod.Context().upload(p)
    assert max(ctx.count_poles(i)[0] for i in range(p.ms.nsubsh)) > 16384
    ctx.run_all(lanczos=True, mixed=mixed)
    assert _check_heap_order(ctx, orc, p.ms.nsubsh, mixed) > 0
    ctx.close()


def test_heap_order_per_channel_calls_and_stable_flag(bdmod, problems, oracle):
    p = problems(6, 20.0, 1, 50)
    orc = oracle(6, 20.0, 1, 50)
    ctx = bdmod.Context().upload(p)
    pv = p.piv
    for ish in range(p.ms.nsubsh):
        ctx.sigma2_build(ish, copy=False)
        ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish])
    assert _check_heap_order(ctx, orc, p.ms.nsubsh, False) > 0
    ctx.run_all(lanczos=True, stable_sort=True)
    assert _check_heap_order(ctx, orc, p.ms.nsubsh, True) > 0
    ctx.close()


def test_sorted_rows_need_a_reduction(bdmod, problems):
    p = problems(4, 20.0, 0, 20)
    ctx = bdmod.Context().upload(p)
    ctx.sigma2_build(0, copy=False)
    with pytest.raises(bdmod.BDError) as e:
        ctx.sigma2_sorted(0)
    assert e.value.code == bdmod.BD_ERR_STATE
    ctx.close()
