"""The reference's file formats (bd_files_*): readers against the synthetic generator's
files, writers byte for byte against the files the reference program itself wrote
(tests/golden/make_file_fixtures.py).  These functions touch no GPU."""
import importlib
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
GOLD = os.path.join(HERE, "golden", "files_nmax2")


@pytest.fixture(scope="module")
def fx(tmp_path_factory):
    mk = importlib.import_module("make_file_fixtures")
    d = str(tmp_path_factory.mktemp("files"))
    paths, prob, counts = mk.inputs(d)
    return dict(paths=paths, prob=prob, counts=counts, mk=mk, dir=d,
                lists=dict(np.load(os.path.join(GOLD, "reference_lists.npz"))))


def _files(bdmod, fx):
    f = bdmod.Files(fx["paths"]["msp"])
    f.read_propagator(fx["paths"]["prop"]).read_pivots(fx["paths"]["piv"])
    return f


def test_readers_return_what_was_written(bdmod, fx):
    p = fx["prob"]
    f = _files(bdmod, fx)
    ms = f.modspace()
    assert ms["nsubsh"] == p.ms.nsubsh and ms["norb"] == p.ms.norb
    for k in ("l", "j2", "ip", "ch", "no", "orb_sh", "orb_n"):
        assert np.array_equal(ms[k], np.asarray(getattr(p.ms, k))), k
    assert np.array_equal(ms["orb_xe"], p.ms.orb_xe)
    assert ms["names"] == list(p.ms.name)
    pr = f.propagator()
    assert pr["nspb"] == p.prop.nspb
    assert np.array_equal(pr["np"], p.prop.np_) and np.array_equal(pr["nh"], p.prop.nh)
    for k in ("ep", "eh", "zp", "zh"):
        assert np.array_equal(pr[k], getattr(p.prop, k)), k
    assert np.array_equal(pr["fqp"], p.prop.fqp) and np.array_equal(pr["fqh"], p.prop.fqh)
    pv = f.pivots()
    assert np.array_equal(pv["npvt"], [len(v) for v in p.piv.vec])
    assert np.array_equal(pv["n_fw"], np.concatenate(p.piv.n_fw)) and np.array_equal(pv["n_bk"], np.concatenate(p.piv.n_bk))
    assert np.array_equal(pv["vec"], np.concatenate([np.asarray(v).reshape(-1) for v in p.piv.vec]))
    f.close()


def test_interaction_lines_kept_and_dropped(bdmod, fx):
    f = _files(bdmod, fx)
    f.read_interaction(fx["paths"]["vpp"], threads=3)
    c = fx["counts"]
    got = f.lines()
    assert got["outside"] == c["outside"] and got["pauli"] == c["pauli"]
    assert got["kept"] == c["lines"] - c["outside"] - c["pauli"]
    f.close()


def test_propagator_and_pivot_writers_match_the_reference(bdmod, fx, tmp_path):
    p = fx["prob"]
    f = _files(bdmod, fx)
    pr = f.propagator()
    out = str(tmp_path / "prop.dat")
    f.write_propagator(out, pr, pr["zp"], pr["zh"])
    assert open(out, "rb").read() == open(os.path.join(GOLD, "prop_written.dat"), "rb").read()
    f.write_propagator(out, pr)            # Z = sum of squared amplitudes: the same here (one-hot)
    assert open(out, "rb").read() == open(os.path.join(GOLD, "prop_written.dat"), "rb").read()
    out2 = str(tmp_path / "piv.dat")
    f.write_pivots(out2, pr, n_fw=5, n_bk=3, z_cut=60.0, zp=pr["zp"], zh=pr["zh"])
    assert open(out2, "rb").read() == open(os.path.join(GOLD, "pivots_written.dat"), "rb").read()
    # the written pivots read back
    g = bdmod.Files(fx["paths"]["msp"]).read_pivots(out2)
    pv = g.pivots()
    assert np.all(pv["n_fw"] == 5) and np.all(pv["n_bk"] == 3)
    f.close(); g.close()


def test_interaction_bin_writer_and_reader(bdmod, fx, tmp_path):
    L = fx["lists"]
    out = str(tmp_path / "vpp.bin")
    bdmod.write_interaction_bin(out, L["vpp_iabJ"], L["vpp_icdJ"], L["vpp_V"], n_alloc=fx["counts"]["lines"])
    assert open(out, "rb").read() == open(os.path.join(GOLD, "vpp_written.bin"), "rb").read()
    f = _files(bdmod, fx)
    f.read_interaction(os.path.join(GOLD, "vpp_written.bin"))
    assert f.lines()["kept"] == len(L["vpp_V"])
    f.close()


@pytest.mark.parametrize("kind", ["plain", "lanczos"])
def test_selfenergy_bin_writer_and_reader(bdmod, fx, tmp_path, kind):
    L = fx["lists"]
    f = _files(bdmod, fx)
    for ish in fx["mk"].CHANNELS:
        name = f.selfenergy_name(os.path.join(GOLD, kind), ish)
        assert os.path.exists(name), name
        r = f.load_selfenergy(name, ish)
        D = int(fx["prob"].ms.no[ish])
        tag = "plain" if kind == "plain" else "lz"
        nden = int(L[f"sig_c{ish}_nden"][1 if kind == "plain" else 0])
        assert r["nden"] == nden
        # (the reference's Lanczos rows of an exhausted chain are NaN: compared as stored)
        assert np.array_equal(r["fw"].reshape(-1), L[f"sig_c{ish}_{tag}_fw"], equal_nan=True)
        assert np.array_equal(r["bk"].reshape(-1), L[f"sig_c{ish}_{tag}_bk"], equal_nan=True)
        ipf = ipb = None
        if kind == "lanczos":
            ipf, ipb = L[f"sig_c{ish}_ipiv_fw"], L[f"sig_c{ish}_ipiv_bk"]
            nu = int(ipf[0])
            assert np.array_equal(r["ipiv_fw"][:nu + 2], ipf[:nu + 2])
        out = str(tmp_path / f"{kind}_{ish}.bin")
        f.save_selfenergy(out, ish, nden, L[f"sig_c{ish}_{tag}_fw"].reshape(-1, nden + D),
                          L[f"sig_c{ish}_{tag}_bk"].reshape(-1, nden + D), ipf, ipb)
        assert open(out, "rb").read() == open(name, "rb").read(), (kind, ish)
    f.close()


def test_malformed_files_are_status_codes(bdmod, tmp_path):
    bad = tmp_path / "bad.dat"
    bad.write_text("# nothing here\n")
    with pytest.raises(bdmod.BDError) as e:
        bdmod.Files(str(bad))
    assert e.value.code == bdmod.BD_ERR_ARG
    with pytest.raises(bdmod.BDError):
        bdmod.Files(str(tmp_path / "missing.dat"))
