"""The C ABI library: it loads without a GPU, exports every symbol include/bd_gb300.h
declares, and reports errors through status codes (no device work is done here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bd_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?(?:int|void|char\s*\*|const char\s*\*)\s*\*?\s*(bd_\w+)\s*\(",
                                 src, re.M)))


def test_header_declarations():
    names = declared()
    for n in ("bd_create", "bd_sigma2_build", "bd_lanczos_reduce", "bd_dyson_solve", "bd_run_all"):
        assert n in names


def test_library_exports_every_declared_symbol(bdmod):
    lib = bdmod.lib()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(bdmod.EXPORTED) <= set(declared())


def test_status_codes_without_device(bdmod):
    lib = bdmod.lib()
    assert lib.bd_version() == 1
    # null context / arguments are rejected before any device call
    assert lib.bd_sync(None) == bdmod.BD_ERR_ARG
    assert lib.bd_run_all(None, 0) == bdmod.BD_ERR_ARG
    assert lib.bd_count_poles(None, 0, None, None) == bdmod.BD_ERR_ARG
    assert lib.bd_last_error(None) == b"null context"


def test_create_reports_missing_device(bdmod):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert bdmod.lib().bd_create(C.byref(h), 0) == bdmod.BD_ERR_CUDA
    assert not h.value
