"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on the CPU."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def synth():
    return importlib.import_module("boccadorata-public_gb300.synth")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    return oracle


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return load


@pytest.fixture(scope="session")
def problems(synth):
    cache = {}

    def get(nmax, hw, seed, nit):
        key = (nmax, hw, seed, nit)
        if key not in cache:
            cache[key] = synth.make_problem(nmax, hw, seed, max(nit, 1))
        return cache[key]
    return get


@pytest.fixture(scope="session")
def oracle(oracle_mod, problems):
    cache = {}

    def get(nmax, hw, seed, nit):
        key = (nmax, hw, seed, nit)
        if key not in cache:
            cache[key] = oracle_mod.Oracle().bind(problems(nmax, hw, seed, nit))
        return cache[key]
    return get


@pytest.fixture(scope="session")
def bdmod():
    return importlib.import_module("boccadorata-public_gb300.bd")


@pytest.fixture(scope="session")
def gpu_ctx(bdmod, problems):
    """One device context per problem (GPU tests only)."""
    cache = {}

    def get(nmax, hw, seed, nit):
        key = (nmax, hw, seed, nit)
        if key not in cache:
            cache[key] = bdmod.Context().upload(problems(nmax, hw, seed, nit))
        return cache[key]
    yield get
    for c in cache.values():
        c.close()
