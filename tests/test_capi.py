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
    return sorted(set(re.findall(r"\b(atm3?_[a-z0-9_]+)\s*\(", src)))


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


def _prototypes():
    """name -> (return type, [parameter types]) parsed from the header."""
    with open(HEADER) as fh:
        src = fh.read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for ret, name, args in re.findall(
            r"^\s*((?:const\s+)?[a-z_]+\s*\**)\s*(atm3?_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src,
            flags=re.M):
        params = [] if args.strip() in ("", "void") else [a.strip() for a in args.split(",")]
        # drop the parameter name, keep the type
        types = [re.sub(r"\s*\b[a-z_0-9]+$", "", a) for a in params]
        out[name] = (ret.replace(" ", ""), [t.replace(" ", "") for t in types])
    return out


def _ctype_of(c):
    P = ctypes.POINTER
    table = {"int": ctypes.c_int, "long": ctypes.c_long, "double": ctypes.c_double,
             "atm_handle": ctypes.c_void_p, "void*": ctypes.c_void_p,
             "atm3_handle": ctypes.c_void_p, "atm3_handle*": P(ctypes.c_void_p),
             "constchar*": ctypes.c_char_p, "int*": P(ctypes.c_int),
             "long*": P(ctypes.c_long), "constint*": P(ctypes.c_int),
             "atm_handle*": P(ctypes.c_void_p), "void**": P(ctypes.c_void_p)}
    return table.get(c)


def test_python_binding_types_match_header():
    """Every ctypes signature in _lib.SIGNATURES has the header's return and
    argument types.  A pointer parameter may also be bound as c_void_p (device
    pointers and numpy buffers handed over as addresses)."""
    from atmospheric_flows_gb300 import _lib

    protos = _prototypes()
    assert sorted(protos) == declared()
    bad = []
    for name, (ret, args) in protos.items():
        res, argtypes = _lib.SIGNATURES[name]
        if len(argtypes) != len(args):
            bad.append((name, "arity", len(args), len(argtypes)))
            continue
        if _ctype_of(ret) is not res:
            bad.append((name, "return", ret, res))
        for i, (c, py) in enumerate(zip(args, argtypes)):
            if "*" in c and py is ctypes.c_void_p:
                ok = True
            elif c in ("double*", "constdouble*"):
                ok = py is ctypes.POINTER(ctypes.c_double)
            elif c == "constdouble*const*":
                ok = py is ctypes.POINTER(ctypes.c_void_p)
            else:
                want = _ctype_of(c)
                ok = want is not None and py is want
            if not ok:
                bad.append((name, i, c, py))
    assert not bad, bad
