"""Write ``oracle_shell_6144_errors.json``: the 3D oracle's errors against the
exact steady solid-body rotation (equation_data.h:57-176), per IMEX step, on
the reference's cell count -- the cubed-sphere shell of 6 x 16 x 16 x 4 =
6144 cells (concentric_hyper_shells refined three times has as many), thin
shell of 10 km, dt 8.64 s, 20 steps.

The reference prints these errors every step (analyze_results,
Atmospheric_Flow.cc:925-985); it cannot run here (deal.II is absent), so the
fixture records the oracle, whose Schur solves reach a true relative residual
of 1e-12 (scaled stopping rule).  The GPU test compares its own errors with
these step by step.

    python tests/golden/make_shell_errors.py      # about 20 minutes on 8 cores
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from atmospheric_flows_gb300.shell import (EARTH_A, ShellParams, build_shell,  # noqa: E402
                                           exact_l2_errors, nodal_to_quad)
from oracle.oracle import OracleShell  # noqa: E402

CFG = dict(n=16, nr=4, thickness=1.0e4, steps=20, eps=1e-12, inner_tol=1e-14)
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_shell_6144_errors.json")


def errors(case, state):
    r, u, p = state
    return exact_l2_errors(case, {"rho": nodal_to_quad(case, r), "u": nodal_to_quad(case, u, 3),
                                  "p": nodal_to_quad(case, p)})


def main():
    case = build_shell(ShellParams(n=CFG["n"], nr=CFG["nr"], r_in=EARTH_A,
                                   r_out=EARTH_A + CFG["thickness"]))
    o = OracleShell(case, eps=CFG["eps"], inner_tol=CFG["inner_tol"], scaled_tol=True,
                    true_residual_check=True)
    hist = [errors(case, o.get_state())]
    t0 = time.time()
    for s in range(CFG["steps"]):
        o.run(1)
        hist.append(errors(case, o.get_state()))
        print(f"step {s + 1} {time.time() - t0:.0f} s {hist[-1]}", flush=True)
    st = o.stats()
    assert st["solve_fail"] == 0
    with open(OUT, "w") as fh:
        json.dump({"config": CFG, "n_cells": case.n_cells, "errors": hist,
                   "stats": {k: int(v) for k, v in st.items()}}, fh, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
