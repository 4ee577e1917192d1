"""Adaptive meshes on the GB300: IMEX steps on a 2:1 mesh with hanging faces
against the oracle, discrete mass conservation through steps and
re-adaptations, and the restrictions of the adaptive path."""
import numpy as np
import pytest

from atmospheric_flows_gb300 import amr
from atmospheric_flows_gb300.hill import HillParams
from oracle.oracle import OracleOperator, OracleSolver

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rl2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def mass(case, rho):
    op = OracleOperator(case)
    op.set_stage(1, 1)
    return op.vmult(rho).sum()


@pytest.mark.parametrize("params,steps", [
    (dict(nx=6, nz=4, degree=3, cfl=2.0, theta_noise=0.1, seed=3), 3),
    (dict(nx=4, nz=3, degree=4, cfl=2.0, periodic=False), 2),
])
def test_amr_steps_match_oracle(cuda_ok, params, steps):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    p = HillParams(**params)
    case = amr.adaptive_case(p, amr.example_tree(p.nx, p.nz, p.periodic))
    assert np.any(case.inner_faces[:, 4] > 0)
    g = EulerSolver(case, eps=1e-12)
    o = OracleSolver(case, eps=1e-12, inner_tol=1e-15)
    g.run(steps)
    o.run(steps)
    for a, b in zip(g.get_state(), o.get_state()):
        assert rl2(a, b) < 1e-10
    assert g.stats()["solve_fail"] == 0
    assert g.stats()["picard_total"] == o.stats()["picard_total"]


def test_adaptive_member_conserves_mass_across_adaptations(cuda_ok):
    p = HillParams(nx=8, nz=4, degree=3, cfl=3.0, theta_noise=0.1, seed=11)
    ap = amr.AdaptParams(max_level=2, every=2)
    m = amr.AdaptiveMember(p, ap, eps=1e-10)
    m0 = mass(m.case, m.case.rho)
    n0 = m.case.n_cells
    assert n0 > p.nx * p.nz  # the initial adaptation refined
    m.run(6)  # two re-adaptations
    assert m.adaptations == 2
    rho, u, pres = m.solver.get_state()
    assert abs(mass(m.case, rho) - m0) / m0 < 1e-12
    st = m.solver.stats()
    assert st["steps"] == 6 and st["solve_fail"] == 0
    assert m.tree.is_balanced()
    d = m.solver.diagnostics()
    assert d["min_rho"] > 0 and np.isfinite(d["max_velocity"])
    m.close()


def test_adaptive_member_is_reproducible(cuda_ok):
    p = HillParams(nx=6, nz=3, degree=2, cfl=3.0, theta_noise=0.1, seed=12)
    out = []
    for _ in range(2):
        m = amr.AdaptiveMember(p, amr.AdaptParams(every=2), eps=1e-10)
        m.run(4)
        out.append(m.solver.get_state())
        m.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def _adaptive(nx=8, nz=4, degree=3, periodic=True, **kw):
    p = HillParams(nx=nx, nz=nz, degree=degree, periodic=periodic, **kw)
    return p, amr.adaptive_case(p, amr.example_tree(p.nx, p.nz, p.periodic))


@pytest.mark.parametrize("precision", [1, 2])
def test_adaptive_vcycle_reduces_residual(cuda_ok, precision):
    """One V-cycle over the adaptive hierarchy (hanging faces on the fine and
    the first coarse levels) reduces the Schur residual of a random vector."""
    import torch

    from atmospheric_flows_gb300.euler_operator import EULEROperator, MatrixFreeStorage

    p, case = _adaptive(cfl=4.0)
    op = EULEROperator(MatrixFreeStorage.from_case(case), case.dt, case.Ma, case.Fr)
    for lv in amr.mg_hierarchy_adaptive(p, case.tree):
        op.add_mg_level(lv)
    rng = np.random.default_rng(3)

    def dev(a):
        return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")

    op.set_rho_for_fixed(dev(case.rho * (1 + 1e-3 * rng.standard_normal(case.rho.shape))))
    op.set_pres_fixed(dev(case.p * (1 + 1e-3 * rng.standard_normal(case.p.shape))))
    op.set_HYPERBOLIC_stage(1)
    op.set_NS_stage(2)
    x = dev(rng.standard_normal(op.n_scalar))
    b = torch.empty_like(x)
    op.vmult(b, x)
    z = torch.empty_like(x)
    op.mg_vcycle(z, b, precision)
    r = torch.empty_like(x)
    op.vmult(r, z)
    red = ((b - r).norm() / b.norm()).item()
    assert red < 0.5, red
    op.close()


@pytest.mark.parametrize("precision,bar", [(1, 1e-8), (2, 1e-10)])
def test_adaptive_multigrid_steps_match_oracle(cuda_ok, precision, bar):
    """IMEX steps on a 2:1 mesh with the multigrid Schur solve (FP32 V-cycle:
    within 1e-8; FP64 V-cycle: within 1e-10 relative L2 per field) against
    the FP64 oracle solving to a true residual of ~1e-13."""
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    p, case = _adaptive(cfl=3.0, theta_noise=0.1, seed=5)
    g = EulerSolver(case, eps=1e-12 if precision == 2 else 1e-10, precision=precision,
                    true_residual_check=True)
    o = OracleSolver(case, eps=1e-13, max_its=3000, inner_tol=1e-15, true_residual_check=True,
                     schur_tol_preconditioned=True)
    g.run(2)
    o.run(2)
    for a, b, name in zip(g.get_state(), o.get_state(), ("rho", "u", "p")):
        assert rl2(a, b) < bar, (name, rl2(a, b))
    st = g.stats()
    assert st["vcycles"] > 0 and st["solve_fail"] == 0
    g.close()


def test_adaptive_member_runs_mixed_precision(cuda_ok):
    """An adaptive member on the mixed-precision multigrid solver re-adapts
    (the hierarchy is rebuilt for each new leaf mesh) and conserves mass."""
    p = HillParams(nx=8, nz=4, degree=3, cfl=3.0, theta_noise=0.1, seed=11)
    m = amr.AdaptiveMember(p, amr.AdaptParams(max_level=2, every=2), eps=1e-10, precision=1)
    m0 = mass(m.case, m.case.rho)
    m.run(4)
    assert m.adaptations == 1
    rho, u, pres = m.solver.get_state()
    assert abs(mass(m.case, rho) - m0) / m0 < 1e-11
    st = m.solver.stats()
    assert st["vcycles"] > 0 and st["solve_fail"] == 0
    m.close()
