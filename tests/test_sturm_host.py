"""The tridiagonal eigenvalue arithmetic of the Dyson eigensolver (csrc/eig_sturm.cuh:
FP32 and double-float Sturm counts in determinant form, Illinois-accelerated
bisection) built for the host with g++ and checked against LAPACK's FP64
eigenvalues on matrices shaped like the Dyson spectra: well separated, degenerate HO
levels with weak couplings, clusters, negligible off-diagonals (splits) and wide
dynamic range.  The device kernels run the same functions; the GPU parity tests
check them end to end."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def sturm_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("sturm") / "sturm_host.so")
    src = os.path.join(HERE, "sturm_host.cpp")
    r = subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", "-o", out, src],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("g++ failed:\n" + r.stderr)
    return C.CDLL(out)


def _eigs(lib, d, e):
    P, I = C.POINTER(C.c_double), C.POINTER(C.c_int)
    n = len(d)
    d = np.ascontiguousarray(d, np.float64)
    e = np.ascontiguousarray(e if len(e) else np.zeros(1), np.float64)
    w, bs, nev = np.zeros(n), np.zeros(n, np.int32), C.c_int()
    lib.bd_sturm_eigenvalues(d.ctypes.data_as(P), e.ctypes.data_as(P), n, w.ctypes.data_as(P),
                             bs.ctypes.data_as(I), C.byref(nev))
    return w, bs, nev.value


def _cases():
    rng = np.random.default_rng(7)
    for n in (1, 2, 3, 7, 40, 94, 257):
        yield n, "separated", rng.normal(size=n) * 50, rng.normal(size=n - 1) * 10
        yield n, "ho-levels", np.round(rng.normal(size=n) * 3) * 16.0, rng.normal(size=n - 1) * 1e-3
        yield n, "constant", np.full(n, 7.0), np.ones(n - 1)
        yield n, "splits", rng.normal(size=n) * 1e3, rng.normal(size=n - 1) * 1e-9 * (rng.random(n - 1) < 0.5)
        yield n, "graded", np.linspace(-100, 300, n), 10 ** rng.uniform(-12, 1, n - 1)
        d = rng.normal(size=n)
        d[::3] = 0.0
        yield n, "zeros", d, rng.normal(size=n - 1) * 1e-6


@pytest.mark.parametrize("n,kind,d,e", list(_cases()), ids=lambda v: str(v) if isinstance(v, (int, str)) else "")
def test_eigenvalues_match_lapack(sturm_lib, n, kind, d, e):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    w, bs, _ = _eigs(sturm_lib, d, e)
    ref = scipy_linalg.eigvalsh_tridiagonal(d, e) if n > 1 else d.copy()
    # stopping rule: width <= max(1e-12 |W|, 1e-13 |T_b|); allow rounding on top
    tn = np.max(np.abs(d)) + 2 * (np.max(np.abs(e)) if n > 1 else 0.0)
    err = np.abs(np.sort(w) - ref)
    assert np.all(err <= 2e-12 * np.abs(ref) + 2e-13 * tn), (kind, float(np.max(err / (np.abs(ref) + tn))))
    # positions are block-major, ascending inside a block
    for b0 in np.unique(bs):
        blk = w[bs == b0]
        assert np.all(np.diff(blk) >= 0)


def test_kac_matrix_eigenvalues(sturm_lib):
    """On a matrix with exact integer eigenvalues (the Kac / Clement matrix:
    d = 0, e_i = sqrt(i (n - i)), eigenvalues -n+1, -n+3, ..., n-1) the eigenvalues
    come out within the stopping rule, max(1e-12 |W|, 1e-13 |T|)."""
    n = 41
    i = np.arange(1, n)
    e = np.sqrt(i * (n - i))
    w, _, nev = _eigs(sturm_lib, np.zeros(n), e)
    exact = np.arange(-(n - 1), n, 2, dtype=np.float64)
    tn = 2.0 * np.max(e)
    assert np.all(np.abs(np.sort(w) - exact) <= 1e-12 * np.abs(exact) + 1e-13 * tn)
    assert nev <= 16 * n   # regula falsi finishes isolated eigenvalues in a few steps
