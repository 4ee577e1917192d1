"""Time-loop parity at the size of the CPU configuration: the flow-over-hill
member of 40x20 cells, Q4, acoustic CFL 5, sponge above 12 km, 200 IMEX steps
(Atmospheric_Flow.cc:1100-1257).

The FP64 oracle's fields after 200 steps are the committed fixture
``tests/golden/oracle_hill_c1_k4.npz`` (tests/golden/make_config1.py; the
oracle needs hours of CPU for them, with its Schur solves at a true relative
residual of ~1e-13).  Bars, relative L2 per field after 200 steps:

* FP64 GPU path -- FGMRES + FP64 multigrid, Schur rtol 1e-12 on the true
  residual: 1e-10;
* mixed precision -- FGMRES + FP32 multigrid, Schur rtol 1e-11: 1e-8.  At
  rtol 1e-10 the mixed path's u drifts to 1.1e-8-1.9e-8 over the 200 steps
  (the Schur residual is amplified into u by dt/Ma^2), so the 1e-8 bar needs
  rtol 1e-11;
* the reference's own solver and tolerance (GMRES + Jacobi on diag(D), eps
  1e-8 on the Jacobi-scaled residual, parameter-file.prm:23): GPU and oracle
  are compared step by step at that setting, live.  They agree to 1e-7 after
  one step and 1e-4 after ten.  That setting is not stable on this member:
  both sides diverge between steps 10 and 50 (the loose implicit solve leaves
  the acoustic terms under-resolved at CFL 5), which the last test records.
"""
import os

import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams, build_case

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "oracle_hill_c1_k4.npz")


def rl2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def config1():
    return build_case(HillParams(nx=40, nz=20, degree=4, cfl=5.0))


@pytest.fixture(scope="module")
def oracle200():
    if not os.path.exists(FIXTURE):
        pytest.fail("missing tests/golden/oracle_hill_c1_k4.npz (tests/golden/make_config1.py)")
    g = np.load(FIXTURE)
    assert int(g["steps"]) == 200 and int(g["solve_fail"]) == 0
    return g


@pytest.mark.parametrize("precision,eps,bar", [(2, 1e-12, 1e-10), (1, 1e-11, 1e-8)],
                         ids=["fp64_multigrid", "mixed_precision"])
def test_200_steps_match_oracle(cuda_ok, config1, oracle200, precision, eps, bar):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    g = EulerSolver(config1, eps=eps, precision=precision, true_residual_check=True)
    g.run(200)
    errs = {name: rl2(a, oracle200[name]) for name, a in zip(("rho", "u", "p"), g.get_state())}
    st = g.stats()
    g.close()
    assert st["steps"] == 200 and st["solve_fail"] == 0
    assert all(e < bar for e in errs.values()), errs


def test_reference_setting_agrees_with_oracle(cuda_ok, config1):
    """GMRES + Jacobi at eps 1e-8 on both sides: the two arms of the headline
    benchmark compute the same fields (1e-7 after 1 step, 1e-4 after 10)."""
    from atmospheric_flows_gb300.euler_solver import EulerSolver
    from oracle.oracle import OracleSolver

    g = EulerSolver(config1, eps=1e-8)
    o = OracleSolver(config1, eps=1e-8)
    done = 0
    for stop, bar in ((1, 1e-7), (10, 1e-4)):
        g.run(stop - done)
        o.run(stop - done)
        done = stop
        for name, a, b in zip(("rho", "u", "p"), g.get_state(), o.get_state()):
            assert rl2(a, b) < bar, (stop, name, rl2(a, b))
    g.close()


def test_reference_setting_diverges_on_this_member(cuda_ok, config1):
    """eps 1e-8 on the Jacobi-scaled residual is too loose for this member at
    CFL 5: the run fails (non-finite or non-converged Schur solve) before
    step 50, while eps 1e-10 runs all 200 steps."""
    from atmospheric_flows_gb300._lib import AtmError
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    g = EulerSolver(config1, eps=1e-8)
    with pytest.raises(AtmError) as ei:
        g.run(50)
    assert ei.value.code in (2, 3)
    assert 10 <= g.stats()["steps"] < 50
    g.close()
    g = EulerSolver(config1, eps=1e-10)
    g.run(200)
    assert all(np.all(np.isfinite(f)) for f in g.get_state())
    g.close()
