"""The double-float arithmetic of the Dyson tridiagonalisation (csrc/df64.cuh: FP32
hi + lo pairs with Knuth's two-sum and the FMA two-product) built for the host with
g++ and checked against FP64: each operation within a few units of 2^-48 of its
operands' scale, and long multiply-add chains (the kernel's sums) accurate too."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("df64") / "df64_host.so")
    r = subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", "-o", out,
                        os.path.join(HERE, "df64_host.cpp")], capture_output=True, text=True)
    if r.returncode != 0:
        pytest.fail("g++ failed:\n" + r.stderr)
    L = C.CDLL(out)
    P = C.POINTER(C.c_double)
    L.bd_df64_ops.argtypes = [C.c_int, P, P, P, C.c_int, P]
    L.bd_df64_sumsq.argtypes = [P, C.c_int]
    L.bd_df64_sumsq.restype = C.c_double
    L.bd_df64_fun.argtypes = [C.c_int, P, C.c_int, P]
    return L


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("op", [0, 1, 2])
def test_operations_to_48_bits(lib, op):
    rng = np.random.default_rng(op)
    n = 20000
    a, b, c = (rng.normal(size=n) * 10 ** rng.uniform(-4, 4, n) for _ in range(3))
    out = np.zeros(n)
    lib.bd_df64_ops(op, _p(a), _p(b), _p(c), n, _p(out))
    ref = [a + b, a * b, a * b + c][op]
    scale = np.maximum.reduce([np.abs(a), np.abs(b), np.abs(c), np.abs(a * b)])
    # the inputs' own double-float rounding is 2^-48 relative, the operation adds a few ulp
    assert np.max(np.abs(out - ref) / scale) < 2.0 ** -44


def test_cancellation_keeps_absolute_accuracy(lib):
    x = np.array([1.0 + 2.0 ** -30, 1e3 + 1e-9, -7.25])
    y = np.array([-1.0, -1e3, 7.25])
    out = np.zeros(3)
    lib.bd_df64_ops(0, _p(x), _p(y), _p(np.zeros(3)), 3, _p(out))
    assert abs(out[0] - 2.0 ** -30) <= 2.0 ** -46
    assert abs(out[1] - 1e-9) <= 1e3 * 2.0 ** -46
    assert out[2] == 0.0


def test_sum_of_squares_chain(lib):
    rng = np.random.default_rng(5)
    a = rng.normal(size=4000) * 30.0
    got = lib.bd_df64_sumsq(_p(a), len(a))
    assert abs(got - float(np.sum(a * a))) <= 1e-13 * float(np.sum(a * a))


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_rsqrt_and_reciprocal(lib, op):
    """Two Newton steps reach double-float rounding; one step (ops 2, 3) squares the
    seed's error: within 2^-42 even from a seed 2 ulp off (the device's rsqrtf)."""
    rng = np.random.default_rng(11 + op)
    a = 10 ** rng.uniform(-12, 12, 5000)
    if op % 2 == 1:
        a *= np.where(rng.random(5000) < 0.5, -1.0, 1.0)
    out = np.zeros_like(a)
    lib.bd_df64_fun(op, _p(a), len(a), _p(out))
    ref = 1.0 / np.sqrt(a) if op % 2 == 0 else 1.0 / a
    assert np.max(np.abs(out / ref - 1.0)) < (2.0 ** -44 if op < 2 else 2.0 ** -42)
