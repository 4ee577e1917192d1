"""The 3D shell path on the GB300 against the 3D oracle: every operator at
1e-12, IMEX steps at 1e-10 (tight solves on both sides), and, on the
reference's cell count (6144 cells), the errors against the reference's known
answer (the exact steady solid-body rotation) step by step as the oracle
gives them."""
import json
import os

import numpy as np
import pytest

from atmospheric_flows_gb300.shell import (EARTH_A, ShellParams, ShellSolver, build_shell,
                                           exact_l2_errors, nodal_to_quad)
from oracle.oracle import OracleShell

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def rl2(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def rotated():
    """Thin shell with every third cell's axes turned: neighbours meet with
    permuted face points."""
    return build_shell(ShellParams(n=4, nr=2, r_in=EARTH_A, r_out=EARTH_A + 1.0e4,
                                   rotate_every=3))


def perturbed(case, seed):
    rng = np.random.default_rng(seed)
    return (case.rho * (1 + 1e-2 * rng.standard_normal(case.rho.shape)),
            case.u + 5.0 * rng.standard_normal(case.u.shape),
            case.p * (1 + 1e-2 * rng.standard_normal(case.p.shape)))


@pytest.mark.parametrize("stage", [1, 2, 3])
def test_rhs_match_oracle(cuda_ok, rotated, stage):
    case = rotated
    g = ShellSolver(case)
    o = OracleShell(case)
    g.set_stage(stage, 1)
    o.set_stage(stage, 1)
    st = [perturbed(case, 10 + j) for j in range(4)]
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    srcs = {
        0: [st[0][0], st[0][1], st[1][0], st[1][1], st[2][0], st[2][1]][:2 * stage],
        1: [x for j in range(stage) for x in st[j]] + ([st[stage][0]] if stage < 3 else []),
        2: [x for j in range(stage) for x in st[j]] + ([st[3][0], st[3][1]] if stage < 3 else
                                                       [st[3][0], st[3][1]]),
    }
    for which, src in srcs.items():
        ns = case.n_cells * 8 * (3 if which == 1 else 1)
        out = torch.empty(ns, dtype=torch.float64, device="cuda")
        g.rhs(which, out, [dev(s) for s in src])
        ref = o.rhs(which, src)
        assert rel(out.cpu().numpy(), ref) < 1e-12, (which, stage)
    g.close()


@pytest.mark.parametrize("ns_stage", [1, 2, 3, 4, 5, 6])
def test_implicit_operators_match_oracle(cuda_ok, rotated, ns_stage):
    case = rotated
    g = ShellSolver(case)
    o = OracleShell(case, inner_tol=1e-15)
    rho, u, p = perturbed(case, 3)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")  # noqa: E731
    g.set_stage(1, ns_stage)
    o.set_stage(1, ns_stage)
    g.set_frozen(rho=dev(rho), pres=dev(p))
    o.set_frozen(rho=rho, p=p)
    ns = case.n_cells * 8
    if ns_stage == 2:
        # B and C alone, then the Schur apply (exact A^{-1} vs the oracle's CG)
        b = torch.empty(3 * ns, dtype=torch.float64, device="cuda")
        g.apply(0, b, dev(p))
        assert rel(b.cpu().numpy(), o.apply(0, p, 3 * ns)) < 1e-12
        cw = torch.empty(ns, dtype=torch.float64, device="cuda")
        g.apply(1, cw, dev(u))
        assert rel(cw.cpu().numpy(), o.apply(1, u, ns)) < 1e-12
    size = 3 * ns if ns_stage in (3, 5) else ns
    src = u if size == 3 * ns else p
    out = torch.empty(size, dtype=torch.float64, device="cuda")
    g.apply(2, out, dev(src))
    assert rel(out.cpu().numpy(), o.apply(2, src, size)) < (1e-11 if ns_stage == 2 else 1e-12)
    g.close()


def test_steps_match_oracle(cuda_ok, rotated):
    """Two IMEX steps with Schur solves to a true residual of ~1e-13 on both
    sides: 1e-10 relative L2 per field."""
    case = rotated
    g = ShellSolver(case, eps=1e-13, max_its=3000, scaled_tol=True, true_residual_check=True)
    o = OracleShell(case, eps=1e-13, inner_tol=1e-15, max_its=3000, scaled_tol=True,
                    true_residual_check=True)
    g.run(2)
    o.run(2)
    for a, b, name in zip(g.get_state(), o.get_state(), ("rho", "u", "p")):
        assert rl2(a, b) < 1e-10, (name, rl2(a, b))
    assert g.stats()["solve_fail"] == 0
    g.close()


FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "oracle_shell_6144_errors.json")


def test_reference_cell_count_follows_the_oracle(cuda_ok):
    """6144 cells (the reference's concentric_hyper_shells refined three
    times has as many), thin shell, 20 steps of 8.64 s.  At every step the
    errors against the exact steady state (what the reference's
    analyze_results prints) equal the oracle's to 1e-6 relative (fixture:
    tests/golden/make_shell_errors.py).  Those errors grow from the
    interpolation level: the Q1 shell's discrete balance is not the exact
    one, and the drift shrinks under refinement (tests/test_shell.py)."""
    with open(FIXTURE) as fh:
        ref = json.load(fh)
    cfg = ref["config"]
    case = build_shell(ShellParams(n=cfg["n"], nr=cfg["nr"], r_in=EARTH_A,
                                   r_out=EARTH_A + cfg["thickness"]))
    assert case.n_cells == ref["n_cells"] == 6144
    g = ShellSolver(case, eps=cfg["eps"], scaled_tol=True, true_residual_check=True)

    def errs(state):
        r, u, p = state
        return exact_l2_errors(case, {"rho": nodal_to_quad(case, r),
                                      "u": nodal_to_quad(case, u, 3), "p": nodal_to_quad(case, p)})

    for step, want in enumerate(ref["errors"]):
        if step:
            g.run(1)
        got = errs(g.get_state())
        for f in ("rho", "u", "p"):
            assert abs(got[f] - want[f]) <= 1e-6 * want[f], (step, f, got[f], want[f])
    assert g.stats()["solve_fail"] == 0
    g.close()
