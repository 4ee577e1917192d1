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


def test_multigrid_rejects_hanging_faces(cuda_ok):
    from atmospheric_flows_gb300._lib import AtmError
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    p = HillParams(nx=8, nz=4, degree=2)
    case = amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))
    with pytest.raises(AtmError):
        EulerSolver(case, precision=1)
    with pytest.raises(ValueError):
        amr.AdaptiveMember(p, precision=1)
