"""Failure detection, injected on the host.

The reference's deal.II solvers throw when a solve does not converge and
``main`` returns 1 (Atmospheric_Flow.cc:1289-1311).  Here every call returns
a status: a Schur solve that reaches its iteration cap ends the step with
NOT_CONVERGED, a non-finite residual with NONFINITE, and a failed step leaves
the state of the last completed step.  The faults are made on the host (a
tiny iteration cap, a NaN written into the uploaded state); no kernel is
made to fault, trap or hang.
"""
import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams, build_case
from atmospheric_flows_gb300.serving import MemberRequest, Server

pytestmark = pytest.mark.gpu

NOT_CONVERGED, NONFINITE = 2, 3


def _case():
    return build_case(HillParams(nx=16, nz=8, degree=3, cfl=4.0))


@pytest.mark.parametrize("precision", [0, 1])
def test_iteration_cap_raises_not_converged(cuda_ok, precision):
    from atmospheric_flows_gb300._lib import AtmError
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    case = _case()
    g = EulerSolver(case, eps=1e-12, max_its=2, precision=precision)
    g.run(0)
    before = g.get_state()
    with pytest.raises(AtmError) as ei:
        g.run(3)
    assert ei.value.code == NOT_CONVERGED
    assert "did not converge" in str(ei.value)
    st = g.stats()
    # the failed step is abandoned: state, clock and step count unchanged
    assert st["steps"] == 0 and st["time"] == 0.0 and st["solve_fail"] == 1
    for a, b in zip(g.get_state(), before):
        assert np.array_equal(a, b)
    g.close()


def test_iteration_cap_can_be_counted_instead(cuda_ok):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    g = EulerSolver(_case(), eps=1e-12, max_its=2, continue_on_not_converged=True)
    g.run(2)
    st = g.stats()
    assert st["steps"] == 2 and st["solve_fail"] > 0
    assert all(np.all(np.isfinite(f)) for f in g.get_state())
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_nan_in_state_raises_nonfinite(cuda_ok, precision):
    from atmospheric_flows_gb300._lib import AtmError
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    case = _case()
    g = EulerSolver(case, eps=1e-10, precision=precision)
    rho = case.rho.copy()
    rho[17] = np.nan
    g.set_state(rho, case.u, case.p)
    with pytest.raises(AtmError) as ei:
        g.run(1)
    assert ei.value.code == NONFINITE
    assert g.stats()["steps"] == 0
    # the context stays usable: a clean state runs again
    g.set_state(case.rho, case.u, case.p)
    g.run(1)
    assert g.stats()["steps"] == 1
    g.close()


def _requests(poison=False):
    p = dict(h0=300.0, u0=8.0, theta_noise=0.1)
    reqs = [MemberRequest(0, 0.0, HillParams(nx=16, nz=8, degree=3, seed=1000, **p), 4),
            MemberRequest(1, 0.0, HillParams(nx=16, nz=8, degree=2, seed=1001, **p), 4),
            MemberRequest(2, 0.0, HillParams(nx=32, nz=16, degree=2, seed=1002, **p), 3)]
    if poison:
        c = build_case(reqs[1].params)
        rho = c.rho.copy()
        rho[5] = np.nan
        reqs[1].initial_state = (rho, c.u, c.p)
    return reqs


def test_poisoned_member_fails_alone(cuda_ok):
    """A member whose uploaded state holds a NaN fails with NONFINITE; the
    members running beside it finish bitwise as they do without it."""
    clean = Server(keep_state=True, chunk_steps=1).run(_requests())
    mixed = Server(keep_state=True, chunk_steps=1).run(_requests(poison=True))
    assert [r.status for r in clean] == ["ok"] * 3
    assert mixed[1].status.startswith("error") and "NONFINITE" in mixed[1].status
    for i in (0, 2):
        assert mixed[i].status == "ok"
        for a, b in zip(clean[i].state, mixed[i].state):
            assert np.array_equal(a, b)
