"""C ABI checks that need no GPU: the library builds, loads, exports every
entry point declared in include/atm_gb300.h, and fails loudly without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "atm_gb300.h")


def declared():
    with open(HEADER) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(atm_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from atmospheric_flows_gb300 import _lib

    return _lib.load()


def test_header_declares_entry_points():
    names = declared()
    assert "atm_ctx_create" in names and "atm_solver_run" in names
    assert len(names) >= 30


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from atmospheric_flows_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == declared()


def test_version_and_error_path(lib):
    assert b"sm_103a" in lib.atm_version()
    # null handle -> BAD_ARG with a message
    assert lib.atm_set_dt(None, 1.0) == 1
    assert b"null handle" in lib.atm_last_error()


def test_no_gpu_fails_loudly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    nodes = np.zeros(18)
    rc = lib.atm_ctx_create(2, 4, 1, 2, nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                            0, None, 0, None, ctypes.byref(h))
    assert rc == 6  # ATM_CUDA_ERROR: there is no CPU path
    assert b"no CPU path" in lib.atm_last_error()
