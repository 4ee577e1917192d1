"""Python mirror of the reference's ``EulerSolver`` (Atmospheric_Flow.cc:57-1257).

The time loop itself runs in the library (C++ host code driving sm_103a
kernels); this class owns the device context, uploads the case and moves
state between host arrays and the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .euler_operator import EULEROperator, MatrixFreeStorage

_dp = ctypes.POINTER(ctypes.c_double)


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


class EulerSolver:
    """IMEX-DG solver for one member (one device context)."""

    REFERENCE_SOLVER = 0  # GMRES + Jacobi on diag(D), as the reference
    PRECISION_MIXED = 1   # FGMRES + FP32 multigrid V-cycle
    PRECISION_FP64_MG = 2  # FGMRES + FP64 multigrid V-cycle

    def __init__(self, case, eps=1e-8, max_its=None, precision=0, dt=None, mg_levels=3,
                 true_residual_check=False, stream=None, levels=None, sponge_target=None,
                 continue_on_not_converged=False, members=None):
        """`levels`: precomputed multigrid levels (default: the hill hierarchy of
        case.params); `sponge_target`: per-node sponge target velocity (batched
        members with different background winds).

        A Schur solve that reaches `max_its` makes :meth:`run` raise
        ``AtmError`` (code NOT_CONVERGED) and leaves the state of the last
        completed step, as the reference's SolverControl throws
        (Atmospheric_Flow.cc:1289-1311); `continue_on_not_converged=True`
        counts it in ``stats()["solve_fail"]`` and carries on instead.

        `members` = (cell offsets, time steps): the case is several
        independent members (batch.concat), each advanced with its own dt and
        its own Krylov and Picard stops; :meth:`member_stats` reports each
        member's outcome (a failed member does not stop the others)."""
        # Krylov iteration cap per Schur solve: the reference's GMRES cap for
        # precision 0; multigrid-preconditioned FGMRES needs tens, so a solve
        # that stalls gives up after 1000 instead of running for minutes
        if max_its is None:
            max_its = 30000 if int(precision) == 0 else 1000
        self.case = case
        self.op = EULEROperator(MatrixFreeStorage.from_case(case))
        self.stream = stream
        if stream is not None:
            _lib.call("atm_set_stream", self.op.handle, ctypes.c_void_p(stream))
        self.dt = case.dt if dt is None else float(dt)
        self.precision = int(precision)
        self.op.set_true_residual_check(true_residual_check)
        if self.precision in (self.PRECISION_MIXED, self.PRECISION_FP64_MG):
            if levels is None:
                if getattr(case, "tree", None) is not None:  # adaptive leaf mesh
                    from .amr import mg_hierarchy_adaptive

                    levels = mg_hierarchy_adaptive(case.params, case.tree, max_levels=mg_levels)
                else:
                    from .hill import mg_hierarchy

                    levels = mg_hierarchy(case.params, max_levels=mg_levels)
            for level in levels:
                self.op.add_mg_level(level)
        _lib.call("atm_solver_init", self.op.handle, self.dt, case.Ma, case.Fr, float(eps),
                  int(max_its), int(precision))
        if continue_on_not_converged:
            _lib.call("atm_solver_set_continue_on_not_converged", self.op.handle, 1)
        self.n_members = 0
        if members is not None:
            off = np.ascontiguousarray(members[0], dtype=np.int32)
            dts = np.ascontiguousarray(members[1], dtype=np.float64)
            if len(off) != len(dts) + 1:
                raise ValueError("members: need len(offsets) == len(dts) + 1")
            _lib.call("atm_set_members", self.op.handle, len(dts),
                      off.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _d(dts))
            self.n_members = len(dts)
        self.n_scalar = self.op.n_scalar
        self.set_state(case.rho, case.u, case.p)
        alpha = np.ascontiguousarray(case.sponge_alpha, dtype=np.float64)
        if np.any(alpha > 0):
            _lib.call("atm_solver_set_sponge", self.op.handle, _d(alpha), case.params.u0, 0.0)
            if sponge_target is not None:
                tgt = np.ascontiguousarray(sponge_target, dtype=np.float64)
                if tgt.shape != (2 * self.n_scalar,):
                    raise ValueError("sponge_target must hold 2 * n_scalar values")
                _lib.call("atm_solver_set_sponge_target", self.op.handle, _d(tgt))

    def set_state(self, rho, u, p):
        r, uu, pp = (np.ascontiguousarray(a, dtype=np.float64) for a in (rho, u, p))
        _lib.call("atm_solver_set_state", self.op.handle, _d(r), _d(uu), _d(pp))

    def get_state(self):
        ns = self.n_scalar
        r, u, p = np.empty(ns), np.empty(2 * ns), np.empty(ns)
        _lib.call("atm_solver_get_state", self.op.handle, _d(r), _d(u), _d(p))
        return r, u, p

    def run(self, n_steps):
        _lib.call("atm_solver_run", self.op.handle, int(n_steps))

    def stats(self):
        s = np.zeros(9)
        _lib.call("atm_solver_stats", self.op.handle, _d(s))
        keys = ("steps", "picard_total", "krylov_total", "picard_stage1", "picard_stage2",
                "solve_fail", "time", "dt", "vcycles")
        return dict(zip(keys, s.tolist()))

    def member_stats(self):
        """Per member: status (0 ok, 2 not converged, 3 non-finite), Picard and
        Krylov iterations, step of its failure (-1 none) and its dt."""
        out = np.zeros(5 * self.n_members)
        _lib.call("atm_member_stats", self.op.handle, self.n_members, _d(out))
        keys = ("status", "picard", "krylov", "fail_step", "dt")
        return [dict(zip(keys, out[5 * m:5 * m + 5].tolist())) for m in range(self.n_members)]

    def diagnostics(self):
        """The printouts of Atmospheric_Flow.cc:1121-1122,1225-1235 for the
        current state: min/max density, max celerity sqrt(gamma p/rho), max
        |u| (device reductions at the nodes), and the Courant numbers
        CFL_c = dt max_c k sqrt(dim) / (Ma h_min), CFL_u = dt max_u k sqrt(dim) / h_min
        with h_min the smallest cell diameter."""
        from .hill import min_cell_diameter

        out = np.zeros(4)
        _lib.call("atm_solver_diagnostics", self.op.handle, _d(out))
        d = dict(zip(("min_rho", "max_rho", "max_celerity", "max_velocity"), out.tolist()))
        if not hasattr(self, "_hmin"):
            self._hmin = min_cell_diameter(self.case.mapping_nodes, self.case.params.mapping_degree)
        scale = self.dt * self.case.degree * np.sqrt(2.0) / self._hmin
        d["cfl_c"] = scale * d["max_celerity"] / self.case.Ma
        d["cfl_u"] = scale * d["max_velocity"]
        return d

    # ------------------------------------------------- checkpoint / restart --
    def save(self, path):
        """Write the state, clock and case parameters to ``path`` (.npz).

        The reference only writes VTU output for visualisation
        (Atmospheric_Flow.cc:885-918); this is a restartable raw dump."""
        import dataclasses

        rho, u, p = self.get_state()
        st = self.stats()
        np.savez(path, rho=rho, u=u, p=p, time=st["time"], steps=int(st["steps"]),
                 dt=self.dt, precision=self.precision,
                 params=np.array(repr(dataclasses.asdict(self.case.params))))

    def load(self, path):
        """Restore a state written by :meth:`save` (same case and mesh)."""
        d = np.load(path)
        n = self.n_scalar
        if d["rho"].shape != (n,) or d["u"].shape != (2 * n,):
            raise ValueError("checkpoint does not match this member's mesh/degree")
        self.set_state(d["rho"], d["u"], d["p"])
        _lib.call("atm_solver_set_clock", self.op.handle, float(d["time"]), int(d["steps"]))

    def close(self):
        self.op.close()
