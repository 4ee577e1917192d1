"""The allocation-free Schur apply (atm_schur_vmult_static_scratch).

It exists for callers that must not have the library allocate device memory
when they call it: a host that owns all HBM through its own pool or admission
budget, or a loop that cannot afford the device-wide synchronisation of
cudaMalloc/cudaFree.  It must give the same S p as the regular entry point
(atm_vmult in NS stage 2), call after call, while its 8 MiB static scratch is
reused.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams, build_case

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _schur_operator(case, seed):
    from atmospheric_flows_gb300.euler_operator import EULEROperator, MatrixFreeStorage

    op = EULEROperator(MatrixFreeStorage.from_case(case), case.dt, case.Ma, case.Fr)
    rng = np.random.default_rng(seed)
    rho = case.rho * (1 + 0.01 * rng.standard_normal(case.rho.shape))
    pf = case.p * (1 + 0.01 * rng.standard_normal(case.p.shape))
    op.set_rho_for_fixed(torch.tensor(rho, device="cuda"))
    op.set_pres_fixed(torch.tensor(pf, device="cuda"))
    op.set_HYPERBOLIC_stage(1)
    op.set_NS_stage(2)
    return op, rng


def _free_device_bytes(L):
    free, total = ctypes.c_double(), ctypes.c_double()
    assert L.atm_device_memory(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def _adaptive_case():
    from atmospheric_flows_gb300 import amr

    p = HillParams(nx=6, nz=4, degree=3, cfl=2.0, theta_noise=0.1, seed=3)
    case = amr.adaptive_case(p, amr.example_tree(p.nx, p.nz, p.periodic))
    assert np.any(case.inner_faces[:, 4] > 0)  # has hanging faces
    return case


@pytest.mark.parametrize("mesh", ["conforming", "adaptive"])
def test_static_scratch_schur_matches_vmult_twice(cuda_ok, mesh):
    """Same S p as atm_vmult (to 1e-12) on three calls in a row, on a
    conforming mesh and on a 2:1 adaptive mesh (the hanging-face kernels).
    The first call of a process may load the library's module holding the
    static array (lazy module loading reserves its 8 MiB then); the calls
    after it change neither the device's free memory nor torch's allocation
    count."""
    from atmospheric_flows_gb300 import _lib

    L = _lib.load()
    case = (build_case(HillParams(nx=8, nz=4, degree=3, cfl=3.0)) if mesh == "conforming"
            else _adaptive_case())
    op, rng = _schur_operator(case, seed=5)
    for call in range(3):
        src = torch.tensor(case.p * (1 + 0.02 * rng.standard_normal(case.p.shape)),
                           device="cuda")
        ref = torch.empty_like(src)
        op.vmult(ref, src)
        out = torch.full_like(src, float("nan"))
        torch.cuda.synchronize()
        free0, alloc0 = _free_device_bytes(L), torch.cuda.memory_allocated()
        rc = L.atm_schur_vmult_static_scratch(op.handle, _p(out), _p(src))
        assert rc == 0, L.atm_last_error()
        torch.cuda.synchronize()
        if call > 0:
            assert _free_device_bytes(L) == free0, f"call {call} changed free device memory"
            assert torch.cuda.memory_allocated() == alloc0
        err = (out - ref).abs().max().item() / ref.abs().max().item()
        assert err < 1e-12, f"call {call}: {err}"
    op.close()


def test_static_scratch_rejects_timing_on(cuda_ok):
    from atmospheric_flows_gb300 import _lib

    L = _lib.load()
    case = build_case(HillParams(nx=8, nz=4, degree=2, cfl=3.0))
    op, _ = _schur_operator(case, seed=7)
    src = torch.tensor(case.p, device="cuda")
    out = torch.empty_like(src)
    assert L.atm_timing_enable(op.handle, 1) == 0
    assert L.atm_schur_vmult_static_scratch(op.handle, _p(out), _p(src)) == 1
    assert b"disable kernel timing" in L.atm_last_error()
    assert L.atm_timing_enable(op.handle, 0) == 0
    assert L.atm_schur_vmult_static_scratch(op.handle, _p(out), _p(src)) == 0
    op.close()


def test_static_scratch_rejects_oversized(cuda_ok):
    from atmospheric_flows_gb300 import _lib

    L = _lib.load()
    # 2 * 336*80*25 = 1,344,000 doubles > 1,048,576
    case = build_case(HillParams(nx=336, nz=80, degree=4, cfl=3.0))
    op, _ = _schur_operator(case, seed=6)
    src = torch.tensor(case.p, device="cuda")
    out = torch.empty_like(src)
    rc = L.atm_schur_vmult_static_scratch(op.handle, _p(out), _p(src))
    assert rc == 1
    assert b"exceeds the static scratch" in L.atm_last_error()
    op.close()
