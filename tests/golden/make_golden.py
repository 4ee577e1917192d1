"""Write the oracle regression fixture ``oracle_hill_k3.npz``.

The reference cannot run here (deal.II is absent), so this fixture records the
oracle itself on a small flow-over-hill member at the time the oracle was
pinned by the analytic tests in tests/test_oracle.py.  It guards the oracle
against silent change; it is not a reference output.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from atmospheric_flows_gb300.hill import HillParams, build_case  # noqa: E402
from oracle.oracle import OracleSolver  # noqa: E402

CFG = dict(nx=8, nz=4, k=3, cfl=3.0, eps=1e-12, inner_tol=1e-15, steps=2)


def main():
    case = build_case(HillParams(nx=CFG["nx"], nz=CFG["nz"], degree=CFG["k"], cfl=CFG["cfl"]))
    s = OracleSolver(case, eps=CFG["eps"], inner_tol=CFG["inner_tol"])
    s.run(CFG["steps"])
    rho, u, p = s.get_state()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_hill_k3.npz")
    np.savez_compressed(out, rho=rho, u=u, p=p, **{k: np.array(v) for k, v in CFG.items()})
    print("wrote", out, s.stats())


if __name__ == "__main__":
    main()
