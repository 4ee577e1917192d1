"""Mesh-table validation of the C ABI on the host (atm_check_mesh, the checks
atm_ctx_create makes before touching the device): valid uniform and 2:1
adaptive tables pass with the right hanging-face count; malformed tables are
refused with ATM_BAD_ARG and a message."""
import ctypes

import numpy as np
import pytest

from atmospheric_flows_gb300 import _lib, amr
from atmospheric_flows_gb300.hill import HillParams, build_case

BAD_ARG = 1


def check(case, inner=None, bdry=None, nodes=None, degree=None):
    lib = _lib.load()
    nodes = np.ascontiguousarray(case.mapping_nodes if nodes is None else nodes, dtype=np.float64)
    inner = np.ascontiguousarray(case.inner_faces if inner is None else inner, dtype=np.int32)
    bdry = np.ascontiguousarray(case.boundary_faces if bdry is None else bdry, dtype=np.int32)
    nh = ctypes.c_int(-1)
    rc = lib.atm_check_mesh(case.degree if degree is None else degree, case.n_cells,
                            case.params.mapping_degree, nodes.ctypes.data, len(inner),
                            inner.ctypes.data, len(bdry), bdry.ctypes.data, ctypes.byref(nh))
    msg = lib.atm_last_error().decode() if rc else ""
    return rc, nh.value, msg


@pytest.fixture(scope="module")
def uniform():
    return build_case(HillParams(nx=6, nz=3, degree=2))


@pytest.fixture(scope="module")
def adaptive():
    p = HillParams(nx=6, nz=4, degree=2)
    return amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))


def test_valid_tables(uniform, adaptive):
    assert check(uniform)[:2] == (0, 0)
    rc, nh, _ = check(adaptive)
    assert rc == 0 and nh == np.count_nonzero(adaptive.inner_faces[:, 4]) // 2 > 0


def test_face_listed_twice(uniform):
    inner = np.concatenate([uniform.inner_faces, uniform.inner_faces[:1]])
    rc, _, msg = check(uniform, inner=inner)
    assert rc == BAD_ARG and "listed twice" in msg


def test_missing_face(uniform):
    rc, _, msg = check(uniform, inner=uniform.inner_faces[1:])
    assert rc == BAD_ARG and "neither an inner nor a boundary face" in msg


def test_out_of_range_and_non_opposite(uniform):
    inner = uniform.inner_faces.copy()
    inner[0, 2] = uniform.n_cells
    assert check(uniform, inner=inner)[0] == BAD_ARG
    inner = uniform.inner_faces.copy()
    inner[0, 3] = inner[0, 1]  # same local face on both sides
    rc, _, msg = check(uniform, inner=inner)
    assert rc == BAD_ARG and "opposite" in msg
    inner = uniform.inner_faces.copy()
    inner[0, 4] = 5
    assert check(uniform, inner=inner)[0] == BAD_ARG


def test_hanging_face_with_one_subface(adaptive):
    inner = adaptive.inner_faces
    first = np.nonzero(inner[:, 4] > 0)[0][0]
    rc, _, msg = check(adaptive, inner=np.delete(inner, first, axis=0))
    assert rc == BAD_ARG
    assert "only one of its two subfaces" in msg or "neither an inner nor a boundary" in msg


def test_inverted_cell_and_bad_degree(uniform):
    nodes = uniform.mapping_nodes.copy()
    nodes[0, :, 1] *= -1.0  # mirror cell 0: negative Jacobian
    rc, _, msg = check(uniform, nodes=nodes)
    assert rc == BAD_ARG and "Jacobian" in msg
    assert check(uniform, degree=6)[0] == BAD_ARG
