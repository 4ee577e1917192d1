"""Host-side case set-up (no GPU): mesh tables, geometry, background state."""
import numpy as np
import pytest

from atmospheric_flows_gb300.hill import (FROUDE, MACH, HillParams, background, build_case,
                                          build_mesh, gll_points, lagrange_matrix)


def test_reference_scaling_constants():
    # parameter-file.prm:7-8
    assert abs(MACH - 0.00357254516) < 1e-11
    assert abs(FROUDE - 0.31933793491) < 1e-11


@pytest.mark.parametrize("periodic", [True, False])
def test_face_tables_cover_every_cell_face_once(periodic):
    p = HillParams(nx=7, nz=3, degree=2, periodic=periodic)
    _, inner, bdry = build_mesh(p)
    seen = {}
    for c0, f0, c1, f1, o in inner:
        assert o == 0
        for key in ((c0, f0), (c1, f1)):
            assert key not in seen
            seen[key] = 1
    for c, f, _ in bdry:
        assert (c, f) not in seen
        seen[(c, f)] = 1
    assert len(seen) == 4 * p.nx * p.nz


def test_conforming_faces():
    # the two sides of every inner face share their mapping nodes
    p = HillParams(nx=6, nz=3, degree=2)
    nodes, inner, _ = build_mesh(p)
    m = p.mapping_degree
    g = nodes.reshape(len(nodes), m + 1, m + 1, 2)

    def side(c, f):
        return {0: g[c, :, 0], 1: g[c, :, m], 2: g[c, 0, :], 3: g[c, m, :]}[f]

    for c0, f0, c1, f1, _ in inner:
        a, b = side(c0, f0), side(c1, f1)
        if f0 == 1 and f1 == 0 and c1 % p.nx == 0:  # periodic wrap: shift by the width
            b = b + np.array([p.x1 - p.x0, 0.0])
        assert np.allclose(a, b, atol=1e-9)


def test_background_hydrostatic():
    p = HillParams()
    z = np.linspace(0, 20000, 2001)
    _, _, pres, rho = background(p, z)
    dpdz = np.gradient(pres, z)
    assert np.max(np.abs(dpdz + 9.80616 * rho) / (9.80616 * rho)) < 1e-3


def test_lagrange_interpolates_nodes():
    for k in range(1, 6):
        x = gll_points(k)
        assert np.allclose(lagrange_matrix(x, x), np.eye(k + 1), atol=1e-13)


def test_case_sizes_and_dt():
    case = build_case(HillParams(nx=40, nz=20, degree=4))
    assert case.n_dofs == 80000
    assert case.rho.shape == (800 * 25,) and case.u.shape == (800 * 50,)
    assert 0.1 < case.dt < 100
    assert np.all(case.sponge_alpha[case.node_xz[..., 1].reshape(-1) <= 12000.0] == 0)
