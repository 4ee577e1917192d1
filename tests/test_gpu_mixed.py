"""Multigrid Schur solve: FP64 FGMRES + geometric multigrid (FP32 or FP64).

Bars: a V-cycle reduces the Schur residual; FGMRES+MG needs far fewer
iterations than GMRES+Jacobi; N IMEX steps with the mixed-precision solve
(rtol 1e-10) stay within 1e-8 relative L2 per field of the FP64 oracle (the
parity bound for the mixed path); the FP64-multigrid path stays within
1e-10.  S is not linear, so all sides solve the Schur equation to its true
residual (the true-residual check) for these comparisons.
"""
import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams, build_case, mg_hierarchy
from oracle.oracle import OracleSolver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def schur_op(case, seed=3):
    from atmospheric_flows_gb300.euler_operator import EULEROperator, MatrixFreeStorage

    op = EULEROperator(MatrixFreeStorage.from_case(case), case.dt, case.Ma, case.Fr)
    for lv in mg_hierarchy(case.params):
        op.add_mg_level(lv)
    rng = np.random.default_rng(seed)
    op.set_rho_for_fixed(dev(case.rho * (1 + 1e-3 * rng.standard_normal(case.rho.shape))))
    op.set_pres_fixed(dev(case.p * (1 + 1e-3 * rng.standard_normal(case.p.shape))))
    op.set_HYPERBOLIC_stage(1)
    op.set_NS_stage(2)
    return op, rng


def tight_oracle(case):
    """FP64 oracle whose Schur solves reach a true relative residual ~1e-12."""
    return OracleSolver(case, eps=1e-13, max_its=3000, inner_tol=1e-15,
                        true_residual_check=True, schur_tol_preconditioned=True)


def test_hierarchy_tables():
    lv = mg_hierarchy(HillParams(nx=40, nz=20))
    assert [l["n_cells"] for l in lv] == [200, 50]
    for l, prev in zip(lv, [40 * 20] + [x["n_cells"] for x in lv]):
        ch = l["children"]
        assert sorted(ch.ravel().tolist()) == list(range(prev))


@pytest.mark.parametrize("k", [2, 4])
@pytest.mark.parametrize("precision", [1, 2])
def test_vcycle_reduces_residual(cuda_ok, k, precision):
    case = build_case(HillParams(nx=32, nz=16, degree=k, cfl=5.0))
    op, rng = schur_op(case)
    x = dev(rng.standard_normal(op.n_scalar))
    b = torch.empty_like(x)
    op.vmult(b, x)
    z = torch.empty_like(x)
    op.mg_vcycle(z, b, precision)
    r = torch.empty_like(x)
    op.vmult(r, z)
    red = ((b - r).norm() / b.norm()).item()
    assert red < 0.5, red


@pytest.mark.parametrize("degree,mapping_degree,bar",
                         [(4, 1, 1e-4), (4, 2, 1e-4), (4, 3, 1e-2), (1, 2, 1e-4), (3, 2, 1e-4),
                          (5, 2, 1e-4)])
def test_fp32_vcycle_follows_the_fp64_vcycle(cuda_ok, degree, mapping_degree, bar):
    """The FP32 levels form their quadrature geometry from the degree-2
    mapping and stage A^{-1} through shared memory: the FP32 V-cycle equals
    the FP64 one to FP32 round-off when the mapping degree is at most 2; at
    degree 3 the FP32 levels see the mapping's degree-2 interpolant, a small
    change of the preconditioner."""
    case = build_case(HillParams(nx=32, nz=16, degree=degree, cfl=5.0,
                                 mapping_degree=mapping_degree))
    op, rng = schur_op(case)
    b = dev(rng.standard_normal(op.n_scalar))
    z1, z2 = torch.empty_like(b), torch.empty_like(b)
    op.mg_vcycle(z1, b, 1)
    op.mg_vcycle(z2, b, 2)
    d = ((z1 - z2).norm() / z2.norm()).item()
    assert d < bar, d
    r = torch.empty_like(b)
    op.vmult(r, z1)
    assert ((b - r).norm() / b.norm()).item() < 0.5


def test_fgmres_beats_jacobi_gmres(cuda_ok):
    case = build_case(HillParams(nx=32, nz=16, degree=4, cfl=5.0))
    op, rng = schur_op(case)
    x_true = dev(case.p * (1 + 1e-3 * rng.standard_normal(case.p.shape)))
    b = torch.empty_like(x_true)
    op.vmult(b, x_true)
    tol = 1e-10 * b.norm().item()
    x1 = dev(case.p)
    c1, it_f, res_f = op.solve_fgmres(x1, b, tol, 500)
    # GMRES + Jacobi stops on the Jacobi-scaled residual: same relative bar
    op.compute_diagonal()
    invd = op.get_matrix_diagonal_inverse()
    x2 = dev(case.p)
    c2, it_g, res_g = op.solve(x2, b, 1e-10 * (invd * b).norm().item(), 2000)
    assert c1 == 0 and c2 == 0
    assert it_f < it_g, (it_f, it_g)
    assert ((x1 - x_true).norm() / x_true.norm()).item() < 1e-6


@pytest.mark.parametrize("params,steps", [
    (dict(nx=16, nz=8, degree=4, cfl=5.0), 3),
    (dict(nx=24, nz=12, degree=3, cfl=5.0, periodic=False), 2),
])
def test_mixed_steps_within_1e8_of_oracle(cuda_ok, params, steps):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    case = build_case(HillParams(**params))
    g = EulerSolver(case, eps=1e-10, precision=1, true_residual_check=True)
    o = tight_oracle(case)
    g.run(steps)
    o.run(steps)
    for a, b, name in zip(g.get_state(), o.get_state(), ("rho", "u", "p")):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 1e-8, (name, err)
    st = g.stats()
    assert st["solve_fail"] == 0 and st["vcycles"] > 0


def test_fp64_multigrid_steps_within_1e10_of_oracle(cuda_ok):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    case = build_case(HillParams(nx=16, nz=8, degree=4, cfl=5.0))
    g = EulerSolver(case, eps=1e-12, precision=2, true_residual_check=True)
    o = tight_oracle(case)
    g.run(3)
    o.run(3)
    for a, b, name in zip(g.get_state(), o.get_state(), ("rho", "u", "p")):
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 1e-10, (name, err)


@pytest.mark.parametrize("precision", [1, 2])
def test_vcycle_graph_replay_is_bitwise_the_launch_sequence(cuda_ok, precision):
    """The captured-graph V-cycle equals the launch-by-launch one bit for bit,
    and is re-captured when the stage coefficient or rho_fix changes."""
    case = build_case(HillParams(nx=16, nz=8, degree=3, cfl=4.0))
    op_g, rng = schur_op(case, seed=5)
    op_e, _ = schur_op(case, seed=5)
    op_e.set_mg_graphs(False)
    b = dev(rng.standard_normal(op_g.n_scalar))
    for stage, new_rho in ((1, False), (1, False), (2, False), (2, True)):
        for op in (op_g, op_e):
            op.set_HYPERBOLIC_stage(stage)
            if new_rho:
                op.set_rho_for_fixed(dev(case.rho * 1.001))
        zg = torch.empty_like(b)
        ze = torch.empty_like(b)
        op_g.mg_vcycle(zg, b, precision)
        op_e.mg_vcycle(ze, b, precision)
        torch.cuda.synchronize()
        assert torch.equal(zg, ze)
    sg, se = op_g.mg_stats(), op_e.mg_stats()
    assert sg["vcycles"] == se["vcycles"] == 4
    assert sg["graph_replays"] == 4 and se["graph_replays"] == 0
