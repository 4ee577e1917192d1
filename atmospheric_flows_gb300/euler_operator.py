"""Python mirror of the reference's ``EULEROperator`` over the C ABI.

Method names, argument order and meaning follow
``EULEROperator<dim, ..., Vec>`` (euler_operator.h:24-211): the setters,
``vmult_rhs_rho_update/velocity_fixed/pressure(dst, src_list)``,
``vmult_pressure`` (B), ``vmult_enthalpy`` (C), ``vmult`` (Base::vmult ->
apply_add per NS stage) and ``compute_diagonal`` /
``get_matrix_diagonal_inverse``.  Vectors are CUDA ``torch.float64``
tensors in the library's cell-contiguous layout; every call runs the sm_103a
kernels of ``libatm_gb300.so`` (there is no CPU path).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _ptr(t) -> ctypes.c_void_p:
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
        raise TypeError("expected a CUDA float64 tensor")
    if not t.is_contiguous():
        raise ValueError("tensor must be contiguous")
    return ctypes.c_void_p(t.data_ptr())


def _np_d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _np_i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class MatrixFreeStorage:
    """Mesh tables + degree: what ``MatrixFree::reinit`` consumes."""

    def __init__(self, degree, n_cells, mapping_degree, mapping_nodes, inner_faces,
                 boundary_faces):
        self.degree = int(degree)
        self.n_cells = int(n_cells)
        self.mapping_degree = int(mapping_degree)
        self.mapping_nodes = mapping_nodes
        self.inner_faces = inner_faces
        self.boundary_faces = boundary_faces

    @classmethod
    def from_case(cls, case):
        return cls(case.degree, case.n_cells, case.params.mapping_degree, case.mapping_nodes,
                   case.inner_faces, case.boundary_faces)


class EULEROperator:
    """GB300 stand-in for ``EULEROperator`` (one device context)."""

    def __init__(self, storage: MatrixFreeStorage, dt=1.0, Mach=1.0, Froude=1.0):
        L = _lib.load()
        nodes, pn = _np_d(storage.mapping_nodes)
        inner, pi = _np_i(storage.inner_faces)
        bdry, pb = _np_i(storage.boundary_faces)
        self._h = ctypes.c_void_p()
        _lib.check(L.atm_ctx_create(2, storage.degree, storage.n_cells, storage.mapping_degree,
                                    pn, len(inner), pi, len(bdry), pb, ctypes.byref(self._h)),
                   "atm_ctx_create")
        self.storage = storage
        self.degree = storage.degree
        self.n_scalar = storage.n_cells * (storage.degree + 1) ** 2
        self.HYPERBOLIC_stage = 1
        self.NS_stage = 1
        self.set_dt(dt)
        self.set_Mach(Mach)
        self.set_Froude(Froude)

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.load().atm_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ setters --
    def set_dt(self, dt):
        _lib.call("atm_set_dt", self._h, float(dt))

    def set_Mach(self, Ma):
        _lib.call("atm_set_mach", self._h, float(Ma))

    def set_Froude(self, Fr):
        _lib.call("atm_set_froude", self._h, float(Fr))

    def set_HYPERBOLIC_stage(self, stage):
        _lib.call("atm_set_hyperbolic_stage", self._h, int(stage))
        self.HYPERBOLIC_stage = int(stage)

    def set_NS_stage(self, stage):
        _lib.call("atm_set_ns_stage", self._h, int(stage))
        self.NS_stage = int(stage)

    def set_rho_for_fixed(self, v):
        _lib.call("atm_set_rho_for_fixed", self._h, _ptr(v))

    def set_pres_fixed(self, v):
        _lib.call("atm_set_pres_fixed", self._h, _ptr(v))

    def set_u_fixed(self, v):
        _lib.call("atm_set_u_fixed", self._h, _ptr(v))

    # ---------------------------------------------------------- operators --
    def _rhs(self, name, dst, src):
        arr = (ctypes.c_void_p * len(src))(*[_ptr(s).value for s in src])
        _lib.call(name, self._h, _ptr(dst), arr, len(src))

    def vmult_rhs_rho_update(self, dst, src):
        self._rhs("atm_vmult_rhs_rho_update", dst, src)

    def vmult_rhs_velocity_fixed(self, dst, src):
        self._rhs("atm_vmult_rhs_velocity_fixed", dst, src)

    def vmult_rhs_pressure(self, dst, src):
        self._rhs("atm_vmult_rhs_pressure", dst, src)

    def vmult_pressure(self, dst, src):
        _lib.call("atm_vmult_pressure", self._h, _ptr(dst), _ptr(src))

    def vmult_enthalpy(self, dst, src):
        _lib.call("atm_vmult_enthalpy", self._h, _ptr(dst), _ptr(src))

    def vmult(self, dst, src):
        _lib.call("atm_vmult", self._h, _ptr(dst), _ptr(src))

    def compute_diagonal(self):
        import torch

        n = self.n_scalar * (2 if self.NS_stage in (3, 5) else 1)
        self._inv_diag = torch.empty(n, dtype=torch.float64, device="cuda")
        _lib.call("atm_diagonal_inverse", self._h, _ptr(self._inv_diag))

    def get_matrix_diagonal_inverse(self):
        return self._inv_diag

    def solve(self, x, b, tol, maxit=30000):
        """Solve op x = b for the current NS stage (x: initial guess, in place).

        Returns (status, iterations, residual); status 2 = not converged."""
        its = ctypes.c_int(0)
        res = ctypes.c_double(0.0)
        code = _lib.load().atm_solve(self._h, _ptr(x), _ptr(b), float(tol), int(maxit),
                                     ctypes.byref(its), ctypes.byref(res))
        if code not in (0, 2):
            _lib.check(code, "atm_solve")
        return code, its.value, res.value

    # ------------------------------------------- mixed-precision multigrid --
    def add_mg_level(self, level):
        """Add the next coarser level (dict from ``hill.mg_hierarchy``)."""
        nodes, pn = _np_d(level["mapping_nodes"])
        inner, pi = _np_i(level["inner_faces"])
        bdry, pb = _np_i(level["boundary_faces"])
        ch, pc = _np_i(level["children"])
        _lib.call("atm_mg_add_level", self._h, int(level["n_cells"]),
                  self.storage.mapping_degree, pn, len(inner), pi, len(bdry), pb, pc)

    def set_mg_smoother(self, degree=4, smoothing_range=15.0, eig_iterations=10,
                        coarse_degree=6):
        _lib.call("atm_mg_set_smoother", self._h, int(degree), float(smoothing_range),
                  int(eig_iterations), int(coarse_degree))

    def mg_vcycle(self, dst, src, precision=1):
        """One V-cycle, FP32 (precision 1) or FP64 (precision 2)."""
        _lib.call("atm_mg_vcycle", self._h, int(precision), _ptr(dst), _ptr(src))

    def set_mg_graphs(self, on):
        """Replay the V-cycle as a captured CUDA graph (default) or not."""
        _lib.call("atm_mg_set_graphs", self._h, int(bool(on)))

    def mg_stats(self):
        out = (ctypes.c_long * 2)()
        _lib.call("atm_mg_stats", self._h, out)
        return {"vcycles": out[0], "graph_replays": out[1]}

    def set_true_residual_check(self, on):
        _lib.call("atm_set_true_residual_check", self._h, int(bool(on)))

    def solve_fgmres(self, x, b, tol, maxit=30000, precision=1):
        its = ctypes.c_int(0)
        res = ctypes.c_double(0.0)
        code = _lib.load().atm_solve_fgmres(self._h, int(precision), _ptr(x), _ptr(b), float(tol),
                                            int(maxit), ctypes.byref(its), ctypes.byref(res))
        if code not in (0, 2):
            _lib.check(code, "atm_solve_fgmres")
        return code, its.value, res.value

    def synchronize(self):
        _lib.call("atm_synchronize", self._h)
