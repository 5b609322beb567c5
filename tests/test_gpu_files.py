"""Problems read from the reference's files and uploaded with bd_upload_files: the
interaction's canonical list is built on the device (keys, radix sort, repeat removal)
and must equal the list the reference program holds after Load_interaction, bit for bit;
the chain's results then equal those of the same problem uploaded from arrays."""
import importlib
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
GOLD = os.path.join(HERE, "golden", "files_nmax2")


def _load(bdmod, paths, vpp_path=None, threads=0):
    f = bdmod.Files(paths["msp"])
    f.read_propagator(paths["prop"]).read_pivots(paths["piv"]).read_interaction(vpp_path or paths["vpp"], threads)
    return f


def test_scrambled_bcd_gives_the_reference_list(bdmod, tmp_path):
    mk = importlib.import_module("make_file_fixtures")
    paths, prob, counts = mk.inputs(str(tmp_path))
    L = dict(np.load(os.path.join(GOLD, "reference_lists.npz")))
    f = _load(bdmod, paths, threads=4)
    ctx = bdmod.Context().upload_files(f, prob)
    a, b, v, rep = ctx.interaction()
    assert np.array_equal(a, L["vpp_iabJ"]) and np.array_equal(b, L["vpp_icdJ"])
    assert np.array_equal(v, L["vpp_V"])
    assert rep == counts["repeated"]
    # the same problem from arrays: identical results
    ctx.run_all(lanczos=True)
    k1 = ctx.koltun_all()
    ref = bdmod.Context().upload(prob)
    ref.run_all(lanczos=True)
    assert np.array_equal(k1, ref.koltun_all())
    f.close(); ctx.close(); ref.close()


@pytest.mark.parametrize("fmt", ["bcd", "bin"])
def test_files_equal_arrays_n_max_4(bdmod, synth, tmp_path, fmt):
    prob = synth.make_problem(4, 20.0, 0, 20)
    paths = synth.write_problem(prob, str(tmp_path))
    if fmt == "bcd":
        vp = str(tmp_path / "vint_scrambled.bcd")
        synth.write_interaction_bcd_scrambled(prob.ms, prob.vpp, vp, seed=3)
    else:
        vp = str(tmp_path / "vint.bin")
        bdmod.write_interaction_bin(vp, prob.vpp.iabJ, prob.vpp.icdJ, prob.vpp.V)
    f = _load(bdmod, paths, vp)
    ctx = bdmod.Context().upload_files(f, prob)
    a, b, v, rep = ctx.interaction()
    assert np.array_equal(a, prob.vpp.iabJ) and np.array_equal(b, prob.vpp.icdJ) and np.array_equal(v, prob.vpp.V)
    ctx.run_all(lanczos=True, mixed=True)
    ref = bdmod.Context().upload(prob)
    ref.run_all(lanczos=True, mixed=True)
    assert np.array_equal(ctx.koltun_all(), ref.koltun_all())
    f.close(); ctx.close(); ref.close()


def test_selfenergy_file_round_trip_into_dyson(bdmod, problems, tmp_path):
    """The ExtSE path (source/BcDor-Main.cpp:350-356): Lanczos rows saved in the reference's
    binary form, loaded back and solved by bd_dyson_rows give the resident solve's result."""
    p = problems(4, 20.0, 0, 20)
    paths = importlib.import_module("boccadorata-public_gb300.synth").write_problem(p, str(tmp_path))
    f = bdmod.Files(paths["msp"])
    ctx = bdmod.Context().upload(p)
    pv = p.piv
    for ish in (0, 5):
        ctx.sigma2_build(ish, copy=False)
        lz = ctx.lanczos_reduce(ish, pv.vec[ish].copy(), pv.n_fw[ish], pv.n_bk[ish])
        D = int(p.ms.no[ish])
        s1 = np.diag(p.ms.orb_xe[p.ms.orb_start[ish]:p.ms.orb_start[ish] + D])
        want = ctx.dyson_solve(ish, s1)
        name = f.selfenergy_name(str(tmp_path), ish)
        f.save_selfenergy(name, ish, lz["NDEN"], lz["lz_fw"], lz["lz_bk"], lz["ipiv_fw"], lz["ipiv_bk"])
        r = f.load_selfenergy(name, ish)
        assert np.array_equal(r["fw"], lz["lz_fw"]) and np.array_equal(r["bk"], lz["lz_bk"])
        got = ctx.dyson_rows(ish, r["nden"], r["fw"], r["bk"], r["ipiv_fw"], r["ipiv_bk"], sig1b=s1)
        np.testing.assert_array_equal(got["koltun"], want["koltun"])
        for tag in ("qp", "qh"):
            assert np.array_equal(got[tag], want[tag]), (ish, tag)
    f.close(); ctx.close()
