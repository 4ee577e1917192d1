"""Ensemble serving: continuous batching of flow-over-hill members on one GPU.

Requests are flow-over-hill members of differing resolution, polynomial
degree and perturbed parameters.  They arrive as a Poisson process and run
under continuous batching:
  * admission by an HBM budget -- a request is admitted as soon as its
    device-memory estimate fits in what the running members leave free;
  * every admitted member owns its device state (context, IMEX stage
    vectors, multigrid hierarchy) for its whole life, and a non-blocking
    CUDA stream driven by its own host thread.  Kernels of all running
    members overlap on the device, and requests that arrive while others run
    join as soon as memory frees up;
  * members advance with the mixed-precision solver (FP64 state, FGMRES
    with an FP32 multigrid preconditioner) unless told otherwise;
  * with batch_size > 1, requests waiting at admission that share the
    degree and the solver are concatenated into one context (batch.py):
    every kernel launch then covers all of their cells, while each member
    keeps its own time step and its own Krylov and Picard stops.  Only small
    members are batched (at most batch_max_cells cells each, 3200 by
    default): their own launches leave most of the GPU idle, while a large
    member fills it alone and, batched, would make its co-residents run its
    Krylov iterations.  A batch runs until its longest member is done; each
    member's result is taken when its own step count is reached, and a
    member that fails is reported alone.

Unbatched members never share device data or reductions, so a member's
result is bitwise the same alone and in a mix (the kernels are
deterministic); a batched member matches its solo run to the solver
tolerance.  The reference has no serving loop; it runs one member per MPI
job (Atmospheric_Flow.cc:1265-1313).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import threading
import time

import numpy as np

from . import _lib
from .batch import batch_key, concat
from .hill import HillParams, build_case

MESHES = ((40, 20), (80, 40), (160, 80), (320, 160))
DEGREES = (2, 3, 4, 5)


@dataclasses.dataclass
class MemberRequest:
    request_id: int
    arrival: float  # seconds after the start of the run
    params: HillParams
    steps: int
    precision: int = 1
    eps: float = 1e-8
    # (rho, u, p) host arrays to start from instead of the case's initial
    # data, e.g. a member resumed from a checkpoint (EulerSolver.save)
    initial_state: tuple | None = None


@dataclasses.dataclass
class MemberResult:
    request_id: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    dofs: int
    status: str
    state: tuple | None = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def make_requests(n=256, rate=4.0, seed=0, meshes=MESHES, degrees=DEGREES,
                  steps_range=(100, 400), steps_scale=1.0, precision=1, eps=1e-8):
    """Requests of the ensemble-serving workload: mesh and degree uniform over
    the given sets, h0 ~ U[100, 600] m, u0 ~ U[5, 15] m/s,
    N ~ U[0.008, 0.012] 1/s, theta' noise 0.1 K seeded with 1000 + id, a
    step count uniform in ``steps_range`` (times ``steps_scale``), Poisson
    arrivals at ``rate`` per second."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        nx, nz = meshes[rng.integers(len(meshes))]
        k = int(degrees[rng.integers(len(degrees))])
        p = HillParams(nx=nx, nz=nz, degree=k, h0=float(rng.uniform(100, 600)),
                       u0=float(rng.uniform(5, 15)), brunt=float(rng.uniform(0.008, 0.012)),
                       theta_noise=0.1, seed=1000 + i)
        steps = max(1, int(round(rng.integers(steps_range[0], steps_range[1] + 1) * steps_scale)))
        out.append(MemberRequest(i, t, p, steps, precision, eps))
    return out


def member_bytes(p: HillParams, precision: int = 1) -> int:
    """Device-memory estimate of one member (context, solver, multigrid)."""
    k = p.degree
    nn2, nq, nc = (k + 1) ** 2, 2 * k + 1, p.nx * p.nz
    ns = nc * nn2
    geo = nc * (5 * nq * nq + 12 * nq) * 8 + nc * 8 * 4 * 2
    blocks = 2 * nc * nn2 * nn2 * 8           # M^{-1}, A^{-1}
    ctx_vec = (4 + 4 + 2 + 1 + 29) * ns * 8   # frozen fields, work, GMRES basis
    solver_vec = (12 + 14) * ns * 8
    total = geo + blocks + ctx_vec + solver_vec
    if precision in (1, 2):
        w = 4 if precision == 1 else 8
        # FGMRES basis + levels (geometry, A^{-1}, vectors) over a 4/3 series
        lv = (nc * (5 * nq * nq + 12 * nq) * w + nc * nn2 * nn2 * w + 10 * ns * w) * 4 // 3
        total += 16 * ns * 8 + lv
    return int(total * 1.15) + (16 << 20)


class Server:
    """Continuous-batching scheduler for ensemble members on one GPU."""

    def __init__(self, hbm_budget=150e9, max_running=32, chunk_steps=10, keep_state=False,
                 batch_size=1, batch_max_cells=3200):
        self.budget = float(hbm_budget)
        self.max_running = int(max_running)
        self.chunk = int(chunk_steps)
        self.keep_state = keep_state
        self.batch_size = int(batch_size)
        self.batch_max_cells = int(batch_max_cells)
        self.batches = []  # member count of every batch started
        self._lock = threading.Condition()
        self._in_use = 0.0
        self._running = 0
        self.results: list[MemberResult] = []
        self.peak_running = 0
        self.peak_bytes = 0.0

    def _run_member(self, req: MemberRequest, t0: float, nbytes: float):
        from .euler_solver import EulerSolver

        admitted = time.perf_counter() - t0
        status = "ok"
        state = None
        stream = ctypes.c_void_p()
        solver = None
        dofs = 0
        try:
            _lib.call("atm_stream_create", ctypes.byref(stream))
            case = build_case(req.params)
            dofs = case.n_dofs
            solver = EulerSolver(case, eps=req.eps, precision=req.precision,
                                 true_residual_check=req.precision != 0,
                                 stream=stream.value)
            if req.initial_state is not None:
                solver.set_state(*req.initial_state)
            left = req.steps
            while left > 0:
                n = min(self.chunk, left)
                solver.run(n)
                left -= n
            if self.keep_state:
                state = solver.get_state()
            else:
                solver.diagnostics()  # one small read-back of the result
        except Exception as exc:  # a failed member must not stop the server
            status = f"error: {exc}"
        finally:
            if solver is not None:
                solver.close()
            if stream.value:
                _lib.call("atm_stream_destroy", stream)
            finished = time.perf_counter() - t0
            with self._lock:
                self._in_use -= nbytes
                self._running -= 1
                self.results.append(MemberResult(req.request_id, req.arrival, admitted, finished,
                                                 req.steps, dofs, status, state))
                self._lock.notify_all()

    def _run_batch(self, reqs, t0: float, nbytes: float):
        from .euler_solver import EulerSolver

        admitted = time.perf_counter() - t0
        n = len(reqs)
        finished = [None] * n
        states = [None] * n
        statuses = ["ok"] * n
        status = "ok"
        stream = ctypes.c_void_p()
        solver = None
        dofs = [0] * n
        try:
            _lib.call("atm_stream_create", ctypes.byref(stream))
            cases = [build_case(r.params) for r in reqs]
            dofs = [c.n_dofs for c in cases]
            b = concat(cases)
            prec = reqs[0].precision
            solver = EulerSolver(b.case, eps=reqs[0].eps, precision=prec,
                                 true_residual_check=prec != 0, stream=stream.value,
                                 levels=b.levels if prec != 0 else None,
                                 sponge_target=b.u_target, members=(b.offsets, b.dts))
            if any(r.initial_state is not None for r in reqs):
                parts = [r.initial_state if r.initial_state is not None else (c.rho, c.u, c.p)
                         for r, c in zip(reqs, cases)]
                solver.set_state(*(np.concatenate([q[f] for q in parts]) for f in range(3)))
            target = [r.steps for r in reqs]
            steps = 0
            while any(f is None for f in finished):
                nxt = min(target[i] for i in range(n) if finished[i] is None)
                k = min(self.chunk, nxt - steps)
                solver.run(k)
                steps += k
                mst = solver.member_stats()
                for i in range(n):
                    if finished[i] is None and mst[i]["status"] != 0:
                        code = _lib.STATUS.get(int(mst[i]["status"]), mst[i]["status"])
                        statuses[i] = (f"error: member failed at step {int(mst[i]['fail_step'])}"
                                       f": {code}")
                        finished[i] = time.perf_counter() - t0
                due = [i for i in range(n) if finished[i] is None and target[i] <= steps]
                if due:
                    parts = b.split_state(solver.get_state()) if self.keep_state else None
                    if parts is None:
                        solver.diagnostics()  # one small read-back per result
                    now = time.perf_counter() - t0
                    for i in due:
                        finished[i] = now
                        if parts is not None:
                            states[i] = tuple(np.array(a) for a in parts[i])
        except Exception as exc:  # a failed batch must not stop the server
            status = f"error: {exc}"
        finally:
            if solver is not None:
                solver.close()
            if stream.value:
                _lib.call("atm_stream_destroy", stream)
            end = time.perf_counter() - t0
            with self._lock:
                self._in_use -= nbytes
                self._running -= 1
                for i, r in enumerate(reqs):
                    self.results.append(MemberResult(
                        r.request_id, r.arrival, admitted,
                        finished[i] if finished[i] is not None else end, r.steps, dofs[i],
                        status if status != "ok" else statuses[i], states[i]))
                self._lock.notify_all()

    def run(self, requests, time_scale=1.0):
        """Serve `requests` (arrival times scaled by `time_scale`); returns
        the results ordered by request id."""
        _lib.load()
        pending = sorted(requests, key=lambda r: r.arrival)
        queue = []  # arrived, not yet admitted (arrival order)
        threads = []
        t0 = time.perf_counter()
        with self._lock:
            while pending or queue:
                now = time.perf_counter() - t0
                while pending and pending[0].arrival * time_scale <= now:
                    queue.append(pending.pop(0))
                if not queue:
                    self._lock.wait(timeout=pending[0].arrival * time_scale - now)
                    continue
                head = queue[0]
                if member_bytes(head.params, head.precision) > self.budget:
                    queue.pop(0)
                    self.results.append(MemberResult(head.request_id, head.arrival, now, now,
                                                     head.steps, 0, "rejected: over budget"))
                    continue
                group = [head]

                def small(r):
                    return r.params.nx * r.params.nz <= self.batch_max_cells

                if self.batch_size > 1 and small(head):
                    key = (batch_key(head.params), head.precision, head.eps)
                    for r in queue[1:]:
                        if len(group) >= self.batch_size:
                            break
                        if small(r) and (batch_key(r.params), r.precision, r.eps) == key:
                            group.append(r)
                nb = sum(member_bytes(r.params, r.precision) for r in group)
                while len(group) > 1 and nb > self.budget:
                    group.pop()
                    nb = sum(member_bytes(r.params, r.precision) for r in group)
                if self._in_use + nb > self.budget or self._running >= self.max_running:
                    self._lock.wait(timeout=0.05)
                    continue
                for r in group:
                    queue.remove(r)
                self._in_use += nb
                self._running += 1
                self.peak_running = max(self.peak_running, self._running)
                self.peak_bytes = max(self.peak_bytes, self._in_use)
                self.batches.append(len(group))
                if len(group) == 1:
                    th = threading.Thread(target=self._run_member, args=(head, t0, nb),
                                          daemon=True)
                else:
                    th = threading.Thread(target=self._run_batch, args=(group, t0, nb),
                                          daemon=True)
                th.start()
                threads.append(th)
        for th in threads:
            th.join()
        self.makespan = time.perf_counter() - t0
        return sorted(self.results, key=lambda r: r.request_id)


def summarize(results, makespan):
    ok = [r for r in results if r.status == "ok"]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    work = sum(r.dofs * r.steps for r in ok)
    return {"requests": len(results), "completed": len(ok),
            "failed": [f"{r.request_id}: {r.status}" for r in results if r.status != "ok"][:5],
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p95_latency_s": float(np.percentile(lat, 95)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_queue_wait_s": float(np.mean([r.admitted - r.arrival for r in ok])) if ok else math.nan,
            "aggregate_dof_steps_per_s": work / makespan if makespan > 0 else math.nan,
            "makespan_s": makespan}
