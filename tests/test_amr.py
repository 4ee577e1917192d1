"""Adaptive meshes with hanging faces: the quadtree, its face tables and
geometry, the solution transfer, and the oracle's discrete identities on
2:1 meshes (no GPU).  The sm_103a kernels on the same meshes are compared
with the oracle in test_gpu_operators.py / test_gpu_amr.py."""
import numpy as np
import pytest

from atmospheric_flows_gb300 import amr
from atmospheric_flows_gb300.hill import HillParams, build_case, build_mesh
from oracle.oracle import OracleOperator


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def perturbed(case, seed=1, amp=0.01):
    rng = np.random.default_rng(seed)
    rho = case.rho * (1 + amp * rng.standard_normal(case.rho.shape))
    u = case.u + 2.0 * rng.standard_normal(case.u.shape)
    p = case.p * (1 + amp * rng.standard_normal(case.p.shape))
    return rho, u, p


@pytest.fixture(scope="module")
def hill_amr():
    p = HillParams(nx=6, nz=4, degree=3, cfl=2.0)
    return amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))


@pytest.fixture(scope="module")
def flat_amr():
    p = HillParams(nx=6, nz=3, degree=3, h0=0.0, cfl=1.0)
    return amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))


def test_balance_and_face_coverage():
    rng = np.random.default_rng(0)
    for periodic in (True, False):
        t = amr.QuadTree(7, 4, periodic, max_level=2)
        for _ in range(3):
            leaves = t.leaves()
            t.refine([leaves[i] for i in rng.choice(len(leaves), 6, replace=False)])
        t.balance()
        assert t.is_balanced()
        inner, bdry = t.face_tables()
        n = len(t.leaves())
        # every cell face appears exactly once, except a coarse hanging face twice
        count = np.zeros((n, 4), dtype=int)
        for c_p, f_p, c_m, f_m, o in inner:
            count[c_p, f_p] += 1
            count[c_m, f_m] += 1
        for c, f, _ in bdry:
            count[c, f] += 1
        coarse = {(c_m, f_m) for c_p, f_p, c_m, f_m, o in inner if o > 0}
        for c in range(n):
            for f in range(4):
                assert count[c, f] == (2 if (c, f) in coarse else 1)
        # both subfaces of every coarse face are listed, with distinct fine cells
        for (c, f) in coarse:
            subs = sorted(o for c_p, f_p, c_m, f_m, o in inner if (c_m, f_m) == (c, f) and o)
            assert subs == [1, 2]


def test_uniform_tree_reproduces_uniform_mesh():
    p = HillParams(nx=5, nz=3, degree=2)
    t = amr.QuadTree(p.nx, p.nz, True)
    inner, bdry = t.face_tables()
    nodes, inner_u, bdry_u = build_mesh(p)
    assert sorted(map(tuple, inner)) == sorted(map(tuple, inner_u))
    assert sorted(map(tuple, bdry)) == sorted(map(tuple, bdry_u))
    assert np.allclose(amr.leaf_mapping_nodes(t, nodes, p.mapping_degree), nodes, atol=1e-9)


def test_hanging_faces_are_geometrically_conforming(hill_amr):
    """The fine face's points coincide with the coarse face's subface points."""
    case = hill_amr
    m = case.params.mapping_degree
    t = np.linspace(0.0, 1.0, 5)
    for c_p, f_p, c_m, f_m, o in case.inner_faces:
        if o == 0:
            continue
        s = o - 1

        def face_pts(cell, f, params):
            pts = np.zeros((len(params), 2))
            ref = [(0.0, z) if f == 0 else (1.0, z) if f == 1 else (z, 0.0) if f == 2 else (z, 1.0)
                   for z in params]
            from atmospheric_flows_gb300.hill import gll_points, lagrange_matrix
            g = gll_points(m)
            X = case.mapping_nodes[cell].reshape(m + 1, m + 1, 2)
            for i, (xi, eta) in enumerate(ref):
                La = lagrange_matrix(g, np.array([xi]))[0]
                Lb = lagrange_matrix(g, np.array([eta]))[0]
                pts[i] = np.einsum("b,a,bad->d", Lb, La, X)
            return pts

        a = face_pts(c_p, f_p, t)
        b = face_pts(c_m, f_m, 0.5 * (t + s))
        if f_p in (0, 1) and abs(a[0, 0] - b[0, 0]) > 1e3:  # periodic seam: shift by the period
            b[:, 0] += np.round((a[0, 0] - b[0, 0]) / 40000.0) * 40000.0
        assert np.max(np.abs(a - b)) < 1e-6


def test_transfer_refine_then_coarsen_is_identity_and_conservative():
    p = HillParams(nx=4, nz=3, degree=3, theta_noise=0.1, seed=5)
    uni = build_case(p)
    base = build_mesh(p)[0]
    t0 = amr.QuadTree(p.nx, p.nz, True)
    t1 = amr.example_tree(p.nx, p.nz)
    nn2 = (p.degree + 1) ** 2
    fields = [uni.rho.reshape(-1, 1, nn2), uni.p.reshape(-1, 1, nn2)]
    fine = amr.transfer_state(t0, t1, base, fields, p.degree, p.mapping_degree)
    back = amr.transfer_state(t1, t0, base, fine, p.degree, p.mapping_degree)
    for a, b in zip(back, fields):
        assert rel(a, b) < 1e-12
    c1 = amr.adaptive_case(p, t1, state=(fine[0].reshape(-1), uni.u, fine[1].reshape(-1)))
    m_uni = OracleOperator(uni)
    m_uni.set_stage(1, 1)
    m_fine = OracleOperator(c1)
    m_fine.set_stage(1, 1)
    m0 = m_uni.vmult(uni.rho).sum()
    assert abs(m_fine.vmult(c1.rho).sum() - m0) / m0 < 1e-13


def test_coarsening_projection_conserves_mass():
    """Children with independent (non-polynomial) data -> parent: the discrete
    mass is the same before and after."""
    p = HillParams(nx=4, nz=3, degree=2, theta_noise=0.1, seed=6)
    base = build_mesh(p)[0]
    t1 = amr.example_tree(p.nx, p.nz)
    c1 = amr.adaptive_case(p, t1)
    rng = np.random.default_rng(2)
    rho = c1.rho * (1 + 0.05 * rng.standard_normal(c1.rho.shape))
    nn2 = (p.degree + 1) ** 2
    t0 = amr.QuadTree(p.nx, p.nz, True)
    coarse = amr.transfer_state(t1, t0, base, [rho.reshape(-1, 1, nn2)], p.degree,
                                p.mapping_degree)[0].reshape(-1)
    o1 = OracleOperator(c1)
    o1.set_stage(1, 1)
    c0 = build_case(p)
    o0 = OracleOperator(c0)
    o0.set_stage(1, 1)
    assert abs(o0.vmult(coarse).sum() - o1.vmult(rho).sum()) / o1.vmult(rho).sum() < 1e-13


@pytest.mark.parametrize("stage", [1, 2, 3])
def test_oracle_rho_rhs_conserves_mass_amr(hill_amr, stage):
    op = OracleOperator(hill_amr)
    op.set_stage(stage, 1)
    rho, u, p = perturbed(hill_amr)
    src = []
    for j in range(stage):
        src += [rho * (1 + 0.1 * j), u * (1 - 0.2 * j)]
    r = op.vmult_rhs_rho_update(src)
    m = op.vmult(rho)
    assert abs(r.sum() - m.sum()) / abs(m.sum()) < 1e-13


def test_oracle_rest_states_amr(hill_amr):
    op = OracleOperator(hill_amr)
    rho, _, p = perturbed(hill_amr)
    z = np.zeros(2 * op.n_scalar)
    op.set_stage(1, 1)
    assert rel(op.vmult_rhs_rho_update([rho, z]), op.vmult(rho)) < 1e-14
    op.set_stage(1, 6)
    assert rel(op.vmult_rhs_pressure([rho, z, p, rho, z]), op.vmult(p)) < 1e-13


def test_oracle_momentum_constant_pressure_amr(flat_amr):
    op = OracleOperator(flat_amr)
    op.set_params(flat_amr.dt, flat_amr.Ma, 1e30)
    n = op.n_scalar
    z = np.zeros(2 * n)
    p = np.full(n, 0.8)
    op.set_stage(1, 3)
    r = op.vmult_rhs_velocity_fixed([np.ones(n), z, p, np.ones(n)])
    scale = flat_amr.dt / flat_amr.Ma ** 2 * 0.8 * 1e4
    assert np.max(np.abs(r)) / scale < 1e-12


def test_oracle_B_C_integration_by_parts_amr(flat_amr):
    op = OracleOperator(flat_amr)
    rng = np.random.default_rng(3)
    n = op.n_scalar
    pf = 0.9
    op.set_pres_fixed(np.full(n, pf))
    for hs in (1, 2):
        op.set_stage(hs, 2)
        q = rng.standard_normal(n)
        w = rng.standard_normal(2 * n)
        lhs = np.dot(op.vmult_pressure(q), w) * flat_amr.Ma ** 2
        rhs = -np.dot(op.vmult_enthalpy(w), q) / (1.4 / 0.4 * pf)
        assert abs(lhs - rhs) / abs(lhs) < 1e-11


def test_indicator_and_marking():
    p = HillParams(nx=8, nz=4, degree=3, theta_noise=0.1, seed=7)
    uni = build_case(p)
    nn2 = (p.degree + 1) ** 2
    ind = amr.theta_perturbation_gradient(p, uni.mapping_nodes, uni.rho.reshape(-1, nn2),
                                          uni.p.reshape(-1, nn2))
    assert ind.shape == (uni.n_cells,) and np.all(ind > 0)
    # without noise the background is hydrostatic with theta' = 0 (up to the
    # interpolation of the background)
    q = HillParams(nx=8, nz=4, degree=3)
    c0 = build_case(q)
    ind0 = amr.theta_perturbation_gradient(q, c0.mapping_nodes, c0.rho.reshape(-1, nn2),
                                           c0.p.reshape(-1, nn2))
    assert np.max(ind0) < 1e-2 * np.min(ind)
    t = amr.QuadTree(p.nx, p.nz, True, 2)
    t1 = amr.mark(t, ind, amr.AdaptParams())
    assert t1.is_balanced()
    # one pass from a uniform mesh: exactly the cells above the 90% quantile
    refined = {iz * p.nx + ix for (l, ix, iz) in t1.refined if l == 0}
    assert refined == set(np.nonzero(ind > np.quantile(ind, 0.9))[0].tolist())
    assert len(t1.leaves()) == p.nx * p.nz + 3 * len(refined)


@pytest.mark.parametrize("k", [1, 2, 4, 5])
def test_oracle_hanging_identities_all_degrees(k):
    """Mass conservation of the rho rhs, the rest states and the B/C
    integration by parts on 2:1 meshes, for every supported degree."""
    p = HillParams(nx=5, nz=3, degree=k, cfl=2.0)
    case = amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))
    op = OracleOperator(case)
    rho, u, pr = perturbed(case, seed=k)
    for stage in (1, 2, 3):
        op.set_stage(stage, 1)
        src = []
        for j in range(stage):
            src += [rho * (1 + 0.1 * j), u * (1 - 0.2 * j)]
        r = op.vmult_rhs_rho_update(src)
        m = op.vmult(rho)
        assert abs(r.sum() - m.sum()) / abs(m.sum()) < 1e-13
    z = np.zeros(2 * op.n_scalar)
    op.set_stage(1, 6)
    assert rel(op.vmult_rhs_pressure([rho, z, pr, rho, z]), op.vmult(pr)) < 1e-13
    flat = HillParams(nx=5, nz=3, degree=k, h0=0.0, cfl=1.0)
    fc = amr.adaptive_case(flat, amr.example_tree(flat.nx, flat.nz))
    of = OracleOperator(fc)
    n = of.n_scalar
    of.set_pres_fixed(np.full(n, 0.9))
    of.set_stage(1, 2)
    rng = np.random.default_rng(k)
    q = rng.standard_normal(n)
    w = rng.standard_normal(2 * n)
    lhs = np.dot(of.vmult_pressure(q), w) * fc.Ma ** 2
    rhs = -np.dot(of.vmult_enthalpy(w), q) / (1.4 / 0.4 * 0.9)
    assert abs(lhs - rhs) / abs(lhs) < 1e-11


@pytest.mark.parametrize("periodic", [True, False])
def test_adaptive_multigrid_hierarchy(periodic):
    """Levels of the multigrid Schur preconditioner on a 2:1 mesh: each level
    merges the finest 2x2 groups of the level above (rows of 4 cells) and
    keeps the rest (rows (cell, -1, -1, -1)), covers every finer cell once,
    passes the library's own table checks (hanging faces included), puts a
    merged cell's children exactly on its four sub-squares, and ends in the
    uniform coarsening of the base mesh."""
    import ctypes

    from atmospheric_flows_gb300 import _lib
    from atmospheric_flows_gb300.hill import gll_points, lagrange_matrix, mg_hierarchy

    L = _lib.load()
    p = HillParams(nx=8, nz=4, degree=2, periodic=periodic)
    tree = amr.example_tree(p.nx, p.nz, p.periodic)
    case = amr.adaptive_case(p, tree)
    levels = amr.mg_hierarchy_adaptive(p, tree)
    m = p.mapping_degree
    n_fine, fine_nodes = case.n_cells, case.mapping_nodes
    merged_levels = 0
    n_adapt, t = 0, amr.coarser_tree(tree)
    while t is not None:
        n_adapt, t = n_adapt + 1, amr.coarser_tree(t)
    assert n_adapt == tree.max_level
    for il, lv in enumerate(levels):
        ch = lv["children"]
        assert ch.shape == (lv["n_cells"], 4)
        same = np.all(ch[:, 1:] < 0, axis=1)
        cells = np.concatenate([ch[same, 0], ch[~same].ravel()])
        assert sorted(cells.tolist()) == list(range(n_fine))  # n_fine: the level above
        assert np.any(~same)
        merged_levels += int(np.any(same))
        nh = ctypes.c_int(-1)
        nodes = np.ascontiguousarray(lv["mapping_nodes"], dtype=np.float64)
        rc = L.atm_check_mesh(p.degree, lv["n_cells"], m,
                              nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                              len(lv["inner_faces"]), lv["inner_faces"].ctypes.data,
                              len(lv["boundary_faces"]), lv["boundary_faces"].ctypes.data,
                              ctypes.byref(nh))
        assert rc == 0, L.atm_last_error()
        n_fine_prev, fine_prev = n_fine, fine_nodes
        n_fine, fine_nodes = lv["n_cells"], nodes
        if il >= n_adapt:
            # uniform coarsening of the base mesh: each level is meshed on the
            # terrain again (as the conforming hierarchy is)
            continue
        # unchanged cells keep their geometry; merged children are sub-squares
        pn = nodes.reshape(-1, m + 1, m + 1, 2)
        fine_nodes_l = fine_prev
        fn = np.asarray(fine_nodes_l).reshape(-1, m + 1, m + 1, 2)
        assert np.array_equal(pn[same], fn[ch[same, 0]])
        ref = gll_points(m)
        for a in range(2):
            for b in range(2):
                La = lagrange_matrix(ref, 0.5 * (a + ref))
                Lb = lagrange_matrix(ref, 0.5 * (b + ref))
                sub = np.einsum("zb,xa,cbad->czxd", Lb, La, pn[~same])
                assert np.allclose(sub, fn[ch[~same, a + 2 * b]], rtol=0, atol=1e-8)
    assert merged_levels == tree.max_level  # the adaptive part keeps cells on each level
    uniform = mg_hierarchy(p)
    assert [lv["n_cells"] for lv in levels[-len(uniform):]] == [u["n_cells"] for u in uniform]
