"""ctypes wrapper of the CPU FP64 oracle (``atm_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline / reference legs of ``bench.py`` -- never by the product
package.  Parity against deal.II is unpinned (deal.II is not installed); the
oracle is pinned by analytic properties in ``tests/test_oracle.py`` and
``tests/test_known_answer.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    src = os.path.join(_HERE, "atm_oracle.cpp")
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "liboracle.so"], check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                 _ip, ctypes.c_int, _ip]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_set_params.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double]
        L.orc_set_stage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc_set_inner_tol.argtypes = [ctypes.c_void_p, ctypes.c_double]
        for n in ("orc_set_rho_for_fixed", "orc_set_pres_fixed", "orc_set_u_fixed"):
            getattr(L, n).argtypes = [ctypes.c_void_p, _dp]
        for n in ("orc_vmult_rhs_rho_update", "orc_vmult_rhs_velocity_fixed",
                  "orc_vmult_rhs_pressure"):
            getattr(L, n).argtypes = [ctypes.c_void_p, _dp, ctypes.POINTER(_dp)]
        for n in ("orc_vmult_pressure", "orc_vmult_enthalpy", "orc_vmult"):
            getattr(L, n).argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_diagonal_inverse.argtypes = [ctypes.c_void_p, _dp]
        L.orc_solve.restype = ctypes.c_int
        L.orc_solve.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_double, ctypes.c_int, _ip]
        L.orc_geometry.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc_basis.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_solver_create.restype = ctypes.c_void_p
        L.orc_solver_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp,
                                        ctypes.c_int, _ip, ctypes.c_int, _ip, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_int]
        L.orc_solver_destroy.argtypes = [ctypes.c_void_p]
        L.orc_solver_set_inner_tol.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_solver_set_true_residual_check.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_set_true_residual_check.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_solver_set_schur_tol_preconditioned.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_solver_set_state.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_solver_get_state.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_solver_set_sponge.argtypes = [ctypes.c_void_p, _dp, ctypes.c_double,
                                            ctypes.c_double]
        L.orc_solver_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_solver_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_long)]
        L.orc_solver_diagnostics.argtypes = [ctypes.c_void_p, _dp]
        L.orc_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def _i(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class OracleOperator:
    """CPU restatement of ``EULEROperator`` (euler_operator.h:24-211)."""

    def __init__(self, case, dt=None):
        L = lib()
        self.case = case
        self.k = case.degree
        self.nn2 = (self.k + 1) ** 2
        self.nc = case.n_cells
        self._nodes = np.ascontiguousarray(case.mapping_nodes, dtype=np.float64)
        self._inner = np.ascontiguousarray(case.inner_faces, dtype=np.int32)
        self._bdry = np.ascontiguousarray(case.boundary_faces, dtype=np.int32)
        self.h = L.orc_create(self.k, self.nc, case.params.mapping_degree, _d(self._nodes),
                              len(self._inner), _i(self._inner), len(self._bdry),
                              _i(self._bdry))
        self.set_params(case.dt if dt is None else dt, case.Ma, case.Fr)
        self.hstage, self.nsstage = 1, 1

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def n_scalar(self):
        return self.nc * self.nn2

    def set_params(self, dt, Ma, Fr):
        lib().orc_set_params(self.h, dt, Ma, Fr)

    def set_stage(self, hyperbolic_stage, ns_stage):
        self.hstage, self.nsstage = hyperbolic_stage, ns_stage
        lib().orc_set_stage(self.h, hyperbolic_stage, ns_stage)

    def set_inner_tol(self, tol):
        lib().orc_set_inner_tol(self.h, tol)

    def set_true_residual_check(self, on):
        lib().orc_set_true_residual_check(self.h, int(bool(on)))

    def set_rho_for_fixed(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_set_rho_for_fixed(self.h, _d(v))

    def set_pres_fixed(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_set_pres_fixed(self.h, _d(v))

    def set_u_fixed(self, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        lib().orc_set_u_fixed(self.h, _d(v))

    def _rhs(self, fn, out_size, src):
        arrs = [np.ascontiguousarray(s, dtype=np.float64) for s in src]
        ptrs = (_dp * len(arrs))(*[_d(a) for a in arrs])
        dst = np.zeros(out_size)
        fn(self.h, _d(dst), ptrs)
        return dst

    def vmult_rhs_rho_update(self, src):
        return self._rhs(lib().orc_vmult_rhs_rho_update, self.n_scalar, src)

    def vmult_rhs_velocity_fixed(self, src):
        return self._rhs(lib().orc_vmult_rhs_velocity_fixed, 2 * self.n_scalar, src)

    def vmult_rhs_pressure(self, src):
        return self._rhs(lib().orc_vmult_rhs_pressure, self.n_scalar, src)

    def _apply(self, fn, out_size, src):
        s = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros(out_size)
        fn(self.h, _d(dst), _d(s))
        return dst

    def vmult_pressure(self, src):
        return self._apply(lib().orc_vmult_pressure, 2 * self.n_scalar, src)

    def vmult_enthalpy(self, src):
        return self._apply(lib().orc_vmult_enthalpy, self.n_scalar, src)

    def _vsize(self):
        return 2 * self.n_scalar if self.nsstage in (3, 5) else self.n_scalar

    def vmult(self, src):
        return self._apply(lib().orc_vmult, self._vsize(), src)

    def diagonal_inverse(self):
        d = np.zeros(self._vsize())
        lib().orc_diagonal_inverse(self.h, _d(d))
        return d

    def solve(self, b, x0=None, tol=1e-14, maxit=10000):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        its = ctypes.c_int(0)
        rc = lib().orc_solve(self.h, _d(x), _d(b), tol, maxit, ctypes.byref(its))
        return x, rc, its.value

    def geometry(self):
        nq2 = (2 * self.k + 1) ** 2
        jxw = np.zeros(self.nc * nq2)
        qx = np.zeros(self.nc * nq2 * 2)
        lib().orc_geometry(self.h, _d(jxw), _d(qx))
        return jxw.reshape(self.nc, nq2), qx.reshape(self.nc, nq2, 2)

    def basis(self):
        nq, nn = 2 * self.k + 1, self.k + 1
        S, D, W = np.zeros(nq * nn), np.zeros(nq * nn), np.zeros(nq)
        lib().orc_basis(self.h, _d(S), _d(D), _d(W))
        return S.reshape(nq, nn), D.reshape(nq, nn), W


class OracleSolver:
    """CPU restatement of ``EulerSolver`` (Atmospheric_Flow.cc:57-1257)."""

    def __init__(self, case, eps=1e-8, max_its=30000, inner_tol=1e-12, dt=None,
                 true_residual_check=False, schur_tol_preconditioned=False):
        L = lib()
        self.case = case
        self._nodes = np.ascontiguousarray(case.mapping_nodes, dtype=np.float64)
        self._inner = np.ascontiguousarray(case.inner_faces, dtype=np.int32)
        self._bdry = np.ascontiguousarray(case.boundary_faces, dtype=np.int32)
        self.h = L.orc_solver_create(case.degree, case.n_cells, case.params.mapping_degree,
                                     _d(self._nodes), len(self._inner), _i(self._inner),
                                     len(self._bdry), _i(self._bdry),
                                     case.dt if dt is None else dt, case.Ma, case.Fr, eps,
                                     max_its)
        L.orc_solver_set_inner_tol(self.h, inner_tol)
        L.orc_solver_set_true_residual_check(self.h, int(bool(true_residual_check)))
        L.orc_solver_set_schur_tol_preconditioned(self.h, int(bool(schur_tol_preconditioned)))
        self.set_state(case.rho, case.u, case.p)
        alpha = np.ascontiguousarray(case.sponge_alpha, dtype=np.float64)
        L.orc_solver_set_sponge(self.h, _d(alpha), case.params.u0, 0.0)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_solver_destroy(self.h)
            self.h = None

    def set_state(self, rho, u, p):
        r, uu, pp = (np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, p))
        lib().orc_solver_set_state(self.h, _d(r), _d(uu), _d(pp))

    def get_state(self):
        ns = self.case.n_cells * (self.case.degree + 1) ** 2
        r, u, p = np.zeros(ns), np.zeros(2 * ns), np.zeros(ns)
        lib().orc_solver_get_state(self.h, _d(r), _d(u), _d(p))
        return r, u, p

    def run(self, n_steps):
        lib().orc_solver_run(self.h, n_steps)

    def diagnostics(self):
        """min/max density, max celerity, max |u| (Atmospheric_Flow.cc:991-1087)."""
        out = np.zeros(4)
        lib().orc_solver_diagnostics(self.h, _d(out))
        return dict(zip(("min_rho", "max_rho", "max_celerity", "max_velocity"), out.tolist()))

    def stats(self):
        out = (ctypes.c_long * 7)()
        lib().orc_solver_stats(self.h, out)
        keys = ("picard_total", "gmres_total", "cg_total", "solve_fail", "inner_cg",
                "picard_stage1", "picard_stage2")
        return dict(zip(keys, list(out)))


def num_threads() -> int:
    return lib().orc_num_threads()


# ---------------------------------------------------------------- 3D shell --
_SHELL = os.path.join(_HERE, "liboracle_shell.so")
_shell = None


def build_shell(force: bool = False) -> str:
    """Compile the 3D shell oracle (shell_oracle.cpp) with the Makefile."""
    src = os.path.join(_HERE, "shell_oracle.cpp")
    if force or not os.path.exists(_SHELL) or os.path.getmtime(_SHELL) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B", "liboracle_shell.so"], check=True)
    return _SHELL


def shell_lib():
    global _shell
    if _shell is None:
        build_shell()
        L = ctypes.CDLL(_SHELL)
        L.orc3_create.restype = ctypes.c_void_p
        L.orc3_create.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, ctypes.c_int, _ip,
                                  ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_double]
        L.orc3_destroy.argtypes = [ctypes.c_void_p]
        L.orc3_set_tolerances.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int]
        L.orc3_set_stage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.orc3_set_frozen.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc3_rhs.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.POINTER(_dp)]
        L.orc3_apply.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc3_set_state.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc3_get_state.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc3_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc3_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_long)]
        _shell = L
    return _shell


class OracleShell:
    """CPU restatement of EULEROperator + EulerSolver in 3D (FE_DGQ(1)) on the
    spherical shell (shell_oracle.cpp); `case` is a shell.ShellCase."""

    def __init__(self, case, eps=1e-8, inner_tol=1e-12, max_its=30000,
                 true_residual_check=False, scaled_tol=False):
        L = shell_lib()
        self.case = case
        self._keep = [np.ascontiguousarray(case.mapping_nodes, dtype=np.float64),
                      np.ascontiguousarray(case.inner_faces, dtype=np.int32),
                      np.ascontiguousarray(case.face_perm, dtype=np.int32),
                      np.ascontiguousarray(case.boundary_faces, dtype=np.int32)]
        nodes, inner, perm, bdry = self._keep
        self.h = L.orc3_create(case.n_cells, _d(nodes), len(inner), _i(inner), _i(perm),
                               len(bdry), _i(bdry), case.dt, case.Ma, case.Fr, eps)
        L.orc3_set_tolerances(self.h, inner_tol, int(bool(true_residual_check)), max_its,
                              int(bool(scaled_tol)))
        self.ns = case.n_cells * 8
        self.set_state(case.rho, case.u, case.p)

    def __del__(self):
        if getattr(self, "h", None):
            shell_lib().orc3_destroy(self.h)
            self.h = None

    def set_stage(self, hyperbolic_stage, ns_stage):
        shell_lib().orc3_set_stage(self.h, hyperbolic_stage, ns_stage)

    def set_frozen(self, rho=None, p=None, u=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (rho, p, u)]
        shell_lib().orc3_set_frozen(self.h, *[None if a is None else _d(a) for a in arrs])

    def rhs(self, which, src):
        """which: 0 rho, 1 momentum, 2 energy; src: the positional source list."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in src]
        ptrs = (_dp * len(arrs))(*[_d(a) for a in arrs])
        dst = np.zeros(self.ns * (3 if which == 1 else 1))
        shell_lib().orc3_rhs(self.h, which, _d(dst), ptrs)
        return dst

    def apply(self, which, src, out_size):
        """which: 0 B, 1 C, 2 vmult of the current NS stage."""
        s = np.ascontiguousarray(src, dtype=np.float64)
        dst = np.zeros(out_size)
        shell_lib().orc3_apply(self.h, which, _d(dst), _d(s))
        return dst

    def set_state(self, rho, u, p):
        r, uu, pp = (np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, p))
        shell_lib().orc3_set_state(self.h, _d(r), _d(uu), _d(pp))

    def get_state(self):
        r, u, p = np.zeros(self.ns), np.zeros(3 * self.ns), np.zeros(self.ns)
        shell_lib().orc3_get_state(self.h, _d(r), _d(u), _d(p))
        return r, u, p

    def run(self, n):
        shell_lib().orc3_run(self.h, n)

    def stats(self):
        out = (ctypes.c_long * 4)()
        shell_lib().orc3_stats(self.h, out)
        return dict(zip(("picard_total", "gmres_total", "solve_fail", "steps"), list(out)))
