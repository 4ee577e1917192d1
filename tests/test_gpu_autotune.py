"""The tile-shape autotuner: the cells-per-block choice changes no result bit,
and its choices are recorded per kernel family, degree and mode."""
import numpy as np
import pytest

from atmospheric_flows_gb300 import _lib
from atmospheric_flows_gb300.hill import HillParams, build_case

pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_autotuned_blocks_give_identical_steps(cuda_ok):
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    # 2304 cells: above the tuning threshold, in a size class no other test uses
    case = build_case(HillParams(nx=64, nz=36, degree=3, cfl=4.0, theta_noise=0.1, seed=2))
    plain = EulerSolver(case, eps=1e-10)
    _lib.call("atm_set_autotune", plain.op.handle, 0)
    plain.run(2)
    tuned = EulerSolver(case, eps=1e-10)
    tuned.run(2)
    for a, b in zip(plain.get_state(), tuned.get_state()):
        assert np.array_equal(a, b)
    rows = [r for r in _lib.autotune_table() if r["degree"] == 3 and r["log2_cells"] == 11]
    fams = {r["family"] for r in rows}
    assert {"rhs_rho", "rhs_vel", "rhs_pres", "B", "CD"} <= fams
    nq = 7
    assert all(r["cells_per_block"] in (64 // nq, 128 // nq, 256 // nq) for r in rows)
    plain.close()
    tuned.close()
