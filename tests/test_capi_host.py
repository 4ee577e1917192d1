"""The C ABI from a compiled C++ host: ``tests/capi_host/host_test.cpp``
includes ``include/atm_gb300.h``, wraps it as the integration guide's
EULEROperator replacement and is built with g++ -Wall -Werror against the
library.  On CPU it validates the mesh tables and checks that a context
cannot be created without a device; on the GPU it applies B and runs one IMEX
step, and both must equal the ctypes binding's results bit for bit."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from atmospheric_flows_gb300 import amr
from atmospheric_flows_gb300.hill import HillParams, build_case

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "capi_host", "host_test.cpp")
PKG = os.path.join(ROOT, "atmospheric_flows_gb300")


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


@pytest.fixture(scope="module")
def host_exe(tmp_path_factory):
    from atmospheric_flows_gb300 import _lib

    _lib.load()  # builds the library if needed
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    cuda = _cuda_home()
    exe = str(tmp_path_factory.mktemp("capi") / "host_test")
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror",
           f"-I{cuda}/include", SRC, "-o", exe, f"-L{PKG}", "-latm_gb300",
           f"-L{cuda}/lib64", "-lcudart", f"-Wl,-rpath,{PKG}:{cuda}/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _cases():
    flat = build_case(HillParams(nx=6, nz=3, degree=3, cfl=3.0))
    p = HillParams(nx=6, nz=4, degree=2, cfl=2.0, theta_noise=0.1, seed=3)
    adaptive = amr.adaptive_case(p, amr.example_tree(p.nx, p.nz, p.periodic))
    return {"conforming": flat, "adaptive": adaptive}


def write_case(case, path):
    k, nc, m = case.degree, case.n_cells, case.params.mapping_degree
    with open(path, "wb") as fh:
        np.array([k, nc, m, len(case.inner_faces), len(case.boundary_faces)],
                 dtype="<i4").tofile(fh)
        np.ascontiguousarray(case.mapping_nodes, dtype="<f8").tofile(fh)
        np.ascontiguousarray(case.inner_faces, dtype="<i4").tofile(fh)
        np.ascontiguousarray(case.boundary_faces, dtype="<i4").tofile(fh)
        np.array([case.dt, case.Ma, case.Fr, case.params.u0], dtype="<f8").tofile(fh)
        for a in (case.rho, case.u, case.p, case.sponge_alpha):
            np.ascontiguousarray(a, dtype="<f8").tofile(fh)


@pytest.mark.parametrize("mesh", ["conforming", "adaptive"])
def test_host_builds_and_checks_tables(host_exe, tmp_path, mesh):
    case = _cases()[mesh]
    path = str(tmp_path / "case.bin")
    write_case(case, path)
    r = subprocess.run([host_exe, path, str(tmp_path / "out.bin"), "cpu"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    nh = int(np.sum(case.inner_faces[:, 4] > 0)) // 2
    assert f"mesh ok: {case.n_cells} cells, {nh} hanging faces" in r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("mesh", ["conforming", "adaptive"])
def test_host_matches_ctypes_binding(cuda_ok, host_exe, tmp_path, mesh):
    import torch

    from atmospheric_flows_gb300.euler_operator import EULEROperator, MatrixFreeStorage
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    case = _cases()[mesh]
    path, out = str(tmp_path / "case.bin"), str(tmp_path / "out.bin")
    write_case(case, path)
    r = subprocess.run([host_exe, path, out, "gpu"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    got = np.fromfile(out, dtype="<f8")
    ns = case.n_cells * (case.degree + 1) ** 2
    assert got.size == 6 * ns
    op = EULEROperator(MatrixFreeStorage.from_case(case), case.dt, case.Ma, case.Fr)
    op.set_HYPERBOLIC_stage(1)
    op.set_NS_stage(2)
    op.set_rho_for_fixed(torch.tensor(case.rho, device="cuda"))
    p = torch.tensor(case.p, device="cuda")
    op.set_pres_fixed(p)
    bp = torch.empty(2 * ns, dtype=torch.float64, device="cuda")
    op.vmult_pressure(bp, p)
    assert np.array_equal(got[:2 * ns], bp.cpu().numpy())
    op.close()
    g = EulerSolver(case, eps=1e-10)
    g.run(1)
    rho, u, pp = g.get_state()
    assert np.array_equal(got[2 * ns:3 * ns], rho)
    assert np.array_equal(got[3 * ns:5 * ns], u)
    assert np.array_equal(got[5 * ns:], pp)
    g.close()
