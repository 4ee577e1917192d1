"""Write ``oracle_hill_c1_k4.npz``: the FP64 oracle after 200 IMEX steps of the
plain flow-over-hill member (40x20 cells, Q4, acoustic CFL 5, sponge above
12 km) -- the CPU configuration of the benchmark suite.

The Schur solves run to a true relative residual of about 1e-13 (GMRES +
Jacobi, eps 1e-13 on the Jacobi-scaled residual, stop only on the recomputed
residual) and the nested A^{-1} and mass solves to 1e-15, so the fields
measure the discretisation and the Picard loop, not solver stopping points.
The oracle needs hours of CPU for this, far too long to run inside a GPU
test; the GPU parity tests compare against this file instead.

    python tests/golden/make_config1.py [--snapshots DIR] [--resume FILE]

``--snapshots DIR`` writes the state every 10 steps into DIR (not committed);
``--resume DIR/c1_stepN.npz`` continues from such a snapshot.  The oracle's
step depends on the state alone (up to the initial guesses of its nested
solves, which move the result by less than their 1e-15 tolerance), so a
resumed run gives the same fields.
"""
import argparse
import os
import re
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from atmospheric_flows_gb300.hill import HillParams, build_case  # noqa: E402
from oracle.oracle import OracleSolver, num_threads  # noqa: E402

CFG = dict(nx=40, nz=20, k=4, cfl=5.0, eps=1e-13, inner_tol=1e-15, max_its=3000, steps=200)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_hill_c1_k4.npz")


def case():
    return build_case(HillParams(nx=CFG["nx"], nz=CFG["nz"], degree=CFG["k"], cfl=CFG["cfl"]))


def tight_solver(c):
    return OracleSolver(c, eps=CFG["eps"], max_its=CFG["max_its"], inner_tol=CFG["inner_tol"],
                        true_residual_check=True, schur_tol_preconditioned=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--snapshots", default=None)
    ap.add_argument("--resume", default=None)
    args = ap.parse_args()
    s = tight_solver(case())
    done, picard, fails = 0, 0, 0
    if args.resume:
        d = np.load(args.resume)
        s.set_state(d["rho"], d["u"], d["p"])
        done = int(re.search(r"step(\d+)", args.resume).group(1))
        picard, fails = int(d["picard_total"]), int(d["solve_fail"])
    t0 = time.time()
    while done < CFG["steps"]:
        n = min(10 - done % 10, CFG["steps"] - done)
        s.run(n)
        done += n
        st = s.stats()
        print(f"step {done}: {time.time() - t0:.0f} s, {st}", flush=True)
        if args.snapshots and done < CFG["steps"]:
            os.makedirs(args.snapshots, exist_ok=True)
            r, u, p = s.get_state()
            np.savez(os.path.join(args.snapshots, f"c1_step{done}.npz"), rho=r, u=u, p=p,
                     picard_total=picard + st["picard_total"],
                     solve_fail=fails + st["solve_fail"])
    rho, u, p = s.get_state()
    st = s.stats()
    np.savez_compressed(OUT, rho=rho, u=u, p=p, picard_total=picard + st["picard_total"],
                        solve_fail=fails + st["solve_fail"], threads=num_threads(),
                        **{k: np.array(v) for k, v in CFG.items()})
    print("wrote", OUT, st)


if __name__ == "__main__":
    main()
