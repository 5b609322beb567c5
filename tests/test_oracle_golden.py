"""The CPU oracle against the golden fixtures written by the reference program itself
(tests/golden/make_golden.py runs oracle/_ref on the same seeded inputs)."""
import numpy as np
import pytest

from helpers import strong_diffs


@pytest.mark.parametrize("name,nmax,seed,nit", [("nmax2_full", 2, 0, 0), ("nmax4_full", 4, 0, 0),
                                                ("nmax4_lanczos20", 4, 0, 20)])
def test_oracle_matches_reference(name, nmax, seed, nit, golden, oracle, problems):
    g = golden(name)
    orc = oracle(nmax, 20.0, seed, nit)
    p = problems(nmax, 20.0, seed, nit)
    keep = set(g["keep"].tolist())
    for ish in range(p.ms.nsubsh):
        r = orc.run_channel(ish, nit > 0)
        assert np.array_equal(r["sig_hf"], g[f"c{ish}_sig_hf"])          # bit-exact
        for tag in ("sig_fw", "sig_bk"):
            a = r[tag]
            chk = np.array([len(a), a.sum(), (a * a).sum(), np.abs(a).max() if len(a) else 0.0])
            assert np.array_equal(chk, g[f"c{ish}_{tag}_sum"])
            if ish in keep:
                assert np.array_equal(a, g[f"c{ish}_{tag}"])
        if ish in keep and nit > 0:
            for tag in ("sorted_fw", "sorted_bk", "lz_fw", "lz_bk"):
                assert np.array_equal(r[tag], g[f"c{ish}_{tag}"]), tag   # reference's single-pass Lanczos, bit-exact
            for tag in ("ipiv_fw", "ipiv_bk"):
                assert np.array_equal(r[tag][:2 + r[tag][0]], g[f"c{ish}_{tag}"][:2 + r[tag][0]])
        for tag in ("qp", "qh"):
            assert len(r[tag]) == int(g[f"c{ish}_{tag}_n"][0])
            e, z = strong_diffs(g[f"c{ish}_{tag}_strong"], r[tag])
            assert e < 1e-10 and z < 1e-9, (ish, tag, e, z)
        np.testing.assert_allclose(r["koltun"], g[f"c{ish}_koltun"], rtol=1e-10, atol=1e-10)


def test_fallback_eigensolver(oracle_mod):
    """The built-in Householder + QL eigensolver of the oracle (used when no LAPACK is
    found), checked against numpy in a fresh process where no LAPACK is registered."""
    import subprocess
    import sys
    code = r"""
import ctypes as C, numpy as np, sys
lib = C.CDLL(sys.argv[1])
assert lib.bdo_has_lapack() == 0
f = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS"); i = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
lib.bdo_dyson.restype = C.c_int
lib.bdo_dyson.argtypes = [C.c_int, C.c_int, f, f, C.c_double, C.c_int, C.c_int, f, C.c_int, i, C.c_int, f,
                          C.c_int, i, f, C.POINTER(C.c_int), C.POINTER(C.c_int), f]
rng = np.random.default_rng(3); n = 40
A = rng.standard_normal((n, n)); A = A + A.T
sol = np.zeros(n * (n + 2)); kol = np.zeros(3); nf, nb = C.c_int(), C.c_int()
z = np.zeros(1); zi = np.zeros(1, np.int32)
rc = lib.bdo_dyson(n, 1, np.ascontiguousarray(A.reshape(-1)), np.zeros(n * n), 1e9, 2, 0, z, 0, zi, 0, z, 0, zi,
                   sol, C.byref(nf), C.byref(nb), kol)
assert rc == 0
w = np.sort(sol.reshape(n, n + 2)[:, 0])
err = np.abs(w - np.linalg.eigvalsh(A)).max()
assert err < 1e-12, err
print("ok", err)
"""
    r = subprocess.run([sys.executable, "-c", code, oracle_mod.PORT_SO], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stderr + r.stdout


def test_oracle_fixtures_of_bench_workloads(golden, oracle):
    """The bench-size oracle fixtures (tests/golden/make_oracle_fixtures.py) are what the
    oracle gives now: a few of the smaller channels recomputed."""
    from helpers import strong_diffs
    for name, key, chans in (("nmax8_lanczos100_oracle", (8, 20.0, 1, 100), (16, 33)),
                             ("nmax10_lanczos100_oracle", (10, 16.0, 2, 100), (20, 41))):
        g = golden(name)
        orc = oracle(*key)
        for ish in chans:
            r = orc.run_channel(ish, True, passes=2)
            assert (len(r["sig_fw"]), len(r["sig_bk"])) == tuple(g[f"c{ish}_counts"])
            np.testing.assert_array_equal(r["koltun"], g[f"c{ish}_koltun"])
            for tag in ("qp", "qh"):
                e, z = strong_diffs(g[f"c{ish}_{tag}_strong"], r[tag][:, :2])
                assert e == 0.0 and z == 0.0, (name, ish, tag)
