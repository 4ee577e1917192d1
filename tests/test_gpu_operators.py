"""Single-operator parity: sm_103a kernels (through the C ABI) vs the FP64 oracle.

Tolerance (single operator application): 1e-12 relative in the max norm,
the parity bar for one vmult.  Schur applies and solves compare at the
solver tolerance they are run to.
"""
import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams, build_case
from oracle.oracle import OracleOperator

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a = a.detach().cpu().numpy() if hasattr(a, "detach") else a
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def dev(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def perturbed(case, seed=1, amp=0.01):
    rng = np.random.default_rng(seed)
    rho = case.rho * (1 + amp * rng.standard_normal(case.rho.shape))
    u = case.u + 2.0 * rng.standard_normal(case.u.shape)
    p = case.p * (1 + amp * rng.standard_normal(case.p.shape))
    return rho, u, p


def states(case, n):
    """n distinct (rho, u, p) states."""
    return [perturbed(case, seed=10 + j, amp=0.01 * (j + 1)) for j in range(n)]


CASES = [
    dict(nx=5, nz=3, degree=1),
    dict(nx=4, nz=3, degree=2),
    dict(nx=4, nz=3, degree=3),
    dict(nx=6, nz=4, degree=4),
    dict(nx=3, nz=2, degree=5),
    dict(nx=4, nz=3, degree=4, periodic=False),
    # 2:1 adaptive meshes with hanging faces (periodic seam, walls, 2 levels)
    dict(nx=6, nz=4, degree=3, amr=True),
    dict(nx=5, nz=3, degree=2, amr=True),
    dict(nx=4, nz=3, degree=4, periodic=False, amr=True),
    dict(nx=4, nz=2, degree=1, amr=True),
    dict(nx=3, nz=2, degree=5, amr=True),
]


def make_case(d):
    d = dict(d)
    adaptive = d.pop("amr", False)
    p = HillParams(cfl=3.0, **d)
    if not adaptive:
        return build_case(p)
    from atmospheric_flows_gb300 import amr

    return amr.adaptive_case(p, amr.example_tree(p.nx, p.nz, p.periodic))


@pytest.fixture(scope="module", params=CASES, ids=lambda d: "k{degree}_{nx}x{nz}".format(**d)
                + ("_walls" if not d.get("periodic", True) else "")
                + ("_amr" if d.get("amr") else ""))
def pair(request, cuda_ok):
    from atmospheric_flows_gb300.euler_operator import EULEROperator, MatrixFreeStorage

    case = make_case(request.param)
    g = EULEROperator(MatrixFreeStorage.from_case(case), case.dt, case.Ma, case.Fr)
    o = OracleOperator(case)
    return case, g, o


def src_lists(case, stage, kind):
    st = states(case, 5)
    rho = [s[0] for s in st]
    u = [s[1] for s in st]
    p = [s[2] for s in st]
    if kind == "rho":
        out = []
        for j in range(stage):
            out += [rho[j], u[j]]
        return out
    if kind == "vel":
        out = []
        for j in range(stage):
            out += [rho[j], u[j], p[j]]
        if stage < 3:
            out += [rho[3]]
        return out
    out = []
    for j in range(stage):
        out += [rho[j], u[j], p[j]]
    return out + [rho[4], u[4]]


@pytest.mark.parametrize("stage", [1, 2, 3])
@pytest.mark.parametrize("kind", ["rho", "vel", "pres"])
def test_explicit_rhs(pair, stage, kind):
    case, g, o = pair
    src = src_lists(case, stage, kind)
    g.set_HYPERBOLIC_stage(stage)
    o.set_stage(stage, 1)
    n = g.n_scalar * (2 if kind == "vel" else 1)
    dst = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    dsrc = [dev(s) for s in src]
    if kind == "rho":
        g.vmult_rhs_rho_update(dst, dsrc)
        ref = o.vmult_rhs_rho_update(src)
    elif kind == "vel":
        g.vmult_rhs_velocity_fixed(dst, dsrc)
        ref = o.vmult_rhs_velocity_fixed(src)
    else:
        g.vmult_rhs_pressure(dst, dsrc)
        ref = o.vmult_rhs_pressure(src)
    torch.cuda.synchronize()
    assert rel(dst, ref) < TOL


@pytest.mark.parametrize("stage", [1, 2])
def test_B_and_C(pair, stage):
    case, g, o = pair
    rho, u, p = perturbed(case, seed=7)
    _, w, pf = perturbed(case, seed=8)
    g.set_HYPERBOLIC_stage(stage)
    o.set_stage(stage, 2)
    g.set_pres_fixed(dev(pf))
    o.set_pres_fixed(pf)
    dB = torch.empty(2 * g.n_scalar, dtype=torch.float64, device="cuda")
    g.vmult_pressure(dB, dev(p))
    assert rel(dB, o.vmult_pressure(p)) < TOL
    dC = torch.empty(g.n_scalar, dtype=torch.float64, device="cuda")
    g.vmult_enthalpy(dC, dev(w))
    assert rel(dC, o.vmult_enthalpy(w)) < TOL


@pytest.mark.parametrize("ns", [1, 3, 4, 5, 6])
def test_mass_vmult_and_diagonal(pair, ns):
    case, g, o = pair
    rho, u, p = perturbed(case, seed=4)
    g.set_rho_for_fixed(dev(rho))
    o.set_rho_for_fixed(rho)
    g.set_NS_stage(ns)
    o.set_stage(1, ns)
    x = u if ns in (3, 5) else p
    dst = torch.empty(len(x), dtype=torch.float64, device="cuda")
    g.vmult(dst, dev(x))
    assert rel(dst, o.vmult(x)) < TOL
    g.compute_diagonal()
    assert rel(g.get_matrix_diagonal_inverse(), o.diagonal_inverse()) < TOL


@pytest.mark.parametrize("stage", [1, 2])
def test_schur_vmult(pair, stage):
    case, g, o = pair
    rho, u, p = perturbed(case, seed=11)
    _, _, pf = perturbed(case, seed=12)
    g.set_HYPERBOLIC_stage(stage)
    g.set_NS_stage(2)
    o.set_stage(stage, 2)
    g.set_rho_for_fixed(dev(rho))
    o.set_rho_for_fixed(rho)
    g.set_pres_fixed(dev(pf))
    o.set_pres_fixed(pf)
    o.set_inner_tol(1e-15)
    dst = torch.empty(g.n_scalar, dtype=torch.float64, device="cuda")
    g.vmult(dst, dev(p))
    # the oracle's A^{-1} is a CG solve (inner tolerance 1e-15 relative)
    assert rel(dst, o.vmult(p)) < 1e-11


@pytest.mark.parametrize("ns", [1, 3, 6])
def test_mass_solves_exact(pair, ns):
    case, g, o = pair
    rho, u, p = perturbed(case, seed=21)
    g.set_rho_for_fixed(dev(rho))
    o.set_rho_for_fixed(rho)
    g.set_NS_stage(ns)
    o.set_stage(1, ns)
    b = o.vmult(u if ns == 3 else p)
    x = torch.zeros(len(b), dtype=torch.float64, device="cuda")
    code, _, _ = g.solve(x, dev(b), 0.0)
    assert code == 0
    ref = u if ns == 3 else p
    assert rel(x, ref) < 1e-11


def test_schur_gmres(pair):
    case, g, o = pair
    rho, u, p = perturbed(case, seed=31)
    _, _, pf = perturbed(case, seed=32)
    g.set_HYPERBOLIC_stage(1)
    g.set_NS_stage(2)
    o.set_stage(1, 2)
    g.set_rho_for_fixed(dev(rho))
    o.set_rho_for_fixed(rho)
    g.set_pres_fixed(dev(pf))
    o.set_pres_fixed(pf)
    o.set_inner_tol(1e-15)
    b = o.vmult(p)
    tol = 1e-13 * np.linalg.norm(b)
    x = dev(0.99 * p)
    code, its, res = g.solve(x, dev(b), tol, 2000)
    xo, rc, its_o = o.solve(b, x0=0.99 * p, tol=tol, maxit=2000)
    assert code == 0 and rc == 0
    assert abs(its - its_o) <= 1
    # S is not linear (the upwind lambda of C depends on A^{-1} B x,
    # euler_operator.h:1497-1498), so GMRES does not return p exactly; the
    # GPU and the oracle run the same Krylov algorithm and must agree.
    assert rel(x, xo) < 1e-10


def test_bad_arguments(pair):
    from atmospheric_flows_gb300._lib import AtmError

    case, g, o = pair
    g.set_HYPERBOLIC_stage(1)
    dst = torch.empty(g.n_scalar, dtype=torch.float64, device="cuda")
    with pytest.raises(AtmError) as e:
        g.vmult_rhs_rho_update(dst, [dst])  # stage 1 needs 2 sources
    assert e.value.code == 1
    with pytest.raises(AtmError):
        g.set_NS_stage(9)
    with pytest.raises(AtmError):
        g.set_dt(-1.0)
