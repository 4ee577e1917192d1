"""Write the oracle regression fixtures ``oracle_hill_k3.npz`` (uniform mesh)
and ``oracle_amr_k2.npz`` (2:1 adaptive mesh with hanging faces).

The reference cannot run here (deal.II is absent), so this fixture records the
oracle itself on a small flow-over-hill member at the time the oracle was
pinned by the analytic tests in tests/test_oracle.py.  It guards the oracle
against silent change; it is not a reference output.

    python tests/golden/make_golden.py

Running it rewrites both files; the uniform fixture in the repository is the
one recorded when the oracle was first pinned (a rerun reproduces it to
~4e-13, the OpenMP and CG ordering).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from atmospheric_flows_gb300 import amr  # noqa: E402
from atmospheric_flows_gb300.hill import HillParams, build_case  # noqa: E402
from oracle.oracle import OracleSolver  # noqa: E402

CFG = dict(nx=8, nz=4, k=3, cfl=3.0, eps=1e-12, inner_tol=1e-15, steps=2)
# adaptive: the fixed 2-level refinement of amr.example_tree, theta' noise
AMR_CFG = dict(nx=6, nz=4, k=2, cfl=3.0, eps=1e-12, inner_tol=1e-15, steps=2, seed=21)


def amr_case(cfg):
    p = HillParams(nx=cfg["nx"], nz=cfg["nz"], degree=cfg["k"], cfl=cfg["cfl"],
                   theta_noise=0.1, seed=cfg["seed"])
    return amr.adaptive_case(p, amr.example_tree(p.nx, p.nz))


def main():
    case = build_case(HillParams(nx=CFG["nx"], nz=CFG["nz"], degree=CFG["k"], cfl=CFG["cfl"]))
    s = OracleSolver(case, eps=CFG["eps"], inner_tol=CFG["inner_tol"])
    s.run(CFG["steps"])
    rho, u, p = s.get_state()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_hill_k3.npz")
    np.savez_compressed(out, rho=rho, u=u, p=p, **{k: np.array(v) for k, v in CFG.items()})
    print("wrote", out, s.stats())
    case = amr_case(AMR_CFG)
    s = OracleSolver(case, eps=AMR_CFG["eps"], inner_tol=AMR_CFG["inner_tol"])
    s.run(AMR_CFG["steps"])
    rho, u, p = s.get_state()
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_amr_k2.npz")
    np.savez_compressed(out, rho=rho, u=u, p=p, **{k: np.array(v) for k, v in AMR_CFG.items()})
    print("wrote", out, s.stats())


if __name__ == "__main__":
    main()
