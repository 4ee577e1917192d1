"""Ensemble serving: request generation and admission (CPU), and on the GPU
the continuous-batching server plus invariance: a member's result is the same
alone and in a mix of concurrently running members."""
import numpy as np
import pytest

from atmospheric_flows_gb300.hill import HillParams
from atmospheric_flows_gb300.serving import (DEGREES, MESHES, MemberRequest, Server,
                                             make_requests, member_bytes, summarize)


def test_request_distribution():
    reqs = make_requests(n=256, rate=8.0, seed=3)
    assert len(reqs) == 256
    arr = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(arr) > 0)
    # Poisson process: mean gap ~ 1/rate
    assert 0.08 < np.mean(np.diff(arr)) < 0.17
    assert {(r.params.nx, r.params.nz) for r in reqs} == set(MESHES)
    assert {r.params.degree for r in reqs} == set(DEGREES)
    assert all(100 <= r.params.h0 <= 600 and 5 <= r.params.u0 <= 15 for r in reqs)
    assert all(0.008 <= r.params.brunt <= 0.012 for r in reqs)
    assert all(100 <= r.steps <= 400 for r in reqs)
    assert reqs[7].params.seed == 1007 and reqs[7].params.theta_noise == 0.1


def test_member_bytes_monotone():
    small = member_bytes(HillParams(nx=40, nz=20, degree=2))
    big = member_bytes(HillParams(nx=320, nz=160, degree=5))
    assert small < big < 10e9


def _fixed_requests():
    p = dict(h0=300.0, u0=8.0, theta_noise=0.1)
    return [MemberRequest(0, 0.0, HillParams(nx=16, nz=8, degree=3, seed=1000, **p), 4),
            MemberRequest(1, 0.0, HillParams(nx=32, nz=16, degree=2, seed=1001, **p), 6),
            MemberRequest(2, 0.0, HillParams(nx=16, nz=8, degree=4, seed=1002, **p), 5)]


@pytest.mark.gpu
def test_member_same_alone_and_in_mix(cuda_ok):
    reqs = _fixed_requests()
    alone = Server(keep_state=True).run([reqs[0]])[0]
    mixed = Server(keep_state=True, chunk_steps=1).run(reqs)
    assert all(r.status == "ok" for r in mixed)
    for a, b in zip(alone.state, mixed[0].state):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_server_budget_and_latency(cuda_ok):
    reqs = make_requests(n=12, rate=50.0, seed=5, meshes=((40, 20), (80, 40)),
                         degrees=(2, 3), steps_range=(2, 4))
    budget = 2.5 * max(member_bytes(r.params) for r in reqs)
    srv = Server(hbm_budget=budget, max_running=8)
    res = srv.run(reqs)
    s = summarize(res, srv.makespan)
    assert s["completed"] == 12, s
    assert srv.peak_bytes <= budget
    assert s["p50_latency_s"] <= s["p95_latency_s"] <= s["p99_latency_s"]
    assert s["aggregate_dof_steps_per_s"] > 0


def _mixed_batch_cases():
    from atmospheric_flows_gb300.hill import build_case

    return [build_case(HillParams(nx=nx, nz=nz, degree=3, h0=h, u0=u, seed=s, theta_noise=0.1,
                                  cfl=cfl))
            for nx, nz, h, u, s, cfl in ((16, 8, 300.0, 8.0, 1, 4.0), (32, 16, 450.0, 12.0, 2, 5.0),
                                         (8, 4, 200.0, 6.0, 3, 3.0))]


def test_batch_tables_are_block_diagonal():
    """Members of different meshes concatenate into disconnected cell ranges;
    each keeps its own dt and wind; the multigrid levels keep members apart,
    and a member whose hierarchy is shallower keeps its coarsest level on
    the deeper levels (rows (cell, -1, -1, -1))."""
    from atmospheric_flows_gb300 import batch

    cases = _mixed_batch_cases()
    b = batch.concat(cases, mg_levels=8)
    off = b.offsets
    assert off == [0, 128, 128 + 512, 128 + 512 + 32]
    assert b.dts == [c.dt for c in cases] and len(set(b.dts)) == 3
    member = lambda cell: np.searchsorted(off, cell, side="right") - 1  # noqa: E731
    inner = b.case.inner_faces
    assert np.all(member(inner[:, 0]) == member(inner[:, 2]))
    assert len(inner) == sum(len(c.inner_faces) for c in cases)
    prev_off = off
    for lv in b.levels:
        ch = lv["children"]
        same = np.all(ch[:, 1:] < 0, axis=1)
        cells = np.concatenate([ch[same, 0], ch[~same].ravel()])
        assert sorted(cells.tolist()) == list(range(prev_off[-1]))
        # every row's cells lie in one member of the finer level
        pm = np.searchsorted(prev_off, ch[:, 0], side="right") - 1
        for q in range(1, 4):
            sel = ch[:, q] >= 0
            assert np.all(np.searchsorted(prev_off, ch[sel, q], side="right") - 1 == pm[sel])
        counts = np.bincount(pm, minlength=3)
        prev_off = [0] + np.cumsum(counts).tolist()
    # the 8x4 member reaches its coarsest level first and is carried along
    assert any(np.all(lv["children"][:, 1:] < 0, axis=1).any() for lv in b.levels)
    tgt = b.u_target.reshape(off[-1], 2, -1)
    assert np.all(tgt[:128, 0] == 8.0) and np.all(tgt[128:640, 0] == 12.0)
    assert np.all(tgt[:, 1] == 0.0)
    rho = b.split(b.case.rho)
    assert all(np.array_equal(r, c.rho) for r, c in zip(rho, cases))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,eps,bar", [(0, 1e-10, 1e-9), (1, 1e-11, 1e-8)])
def test_member_same_alone_and_in_batch(cuda_ok, precision, eps, bar):
    """Three members of different meshes and time steps in one context: each
    matches its solo run at its own dt -- GMRES + Jacobi to 1e-9, FGMRES +
    FP32 multigrid to 1e-8 relative L2 per field (the batch's V-cycle uses
    the batch's Chebyshev interval, so the preconditioner differs)."""
    from atmospheric_flows_gb300 import batch
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    cases = _mixed_batch_cases()
    # 5 levels: the 8x4 member's hierarchy (3 levels) is padded on the deeper ones
    b = batch.concat(cases, mg_levels=5)
    kw = dict(eps=eps, precision=precision, true_residual_check=precision != 0, mg_levels=5)
    g = EulerSolver(b.case, levels=b.levels if precision else None, sponge_target=b.u_target,
                    members=(b.offsets, b.dts), **kw)
    g.run(3)
    parts = b.split_state(g.get_state())
    ms = g.member_stats()
    g.close()
    assert [m["status"] for m in ms] == [0, 0, 0]
    for i, c in enumerate(cases):
        s = EulerSolver(c, **kw)
        s.run(3)
        st = s.stats()
        for a, ref in zip(parts[i], s.get_state()):
            assert np.linalg.norm(a - ref) / np.linalg.norm(ref) < bar
        if precision == 0:
            assert ms[i]["picard"] == st["picard_total"]
        s.close()


@pytest.mark.gpu
def test_poisoned_member_fails_alone_in_batch(cuda_ok):
    """A batched member whose state holds a NaN fails alone (NONFINITE, at
    step 1); the other members of the same context are bitwise what they are
    beside a clean member."""
    from atmospheric_flows_gb300 import batch
    from atmospheric_flows_gb300.euler_solver import EulerSolver

    cases = _mixed_batch_cases()
    b = batch.concat(cases)
    out = []
    for poison in (False, True):
        g = EulerSolver(b.case, eps=1e-10, sponge_target=b.u_target, members=(b.offsets, b.dts))
        rho = b.case.rho.copy()
        if poison:
            rho[b.offsets[1] * 16 + 7] = np.nan
        g.set_state(rho, b.case.u, b.case.p)
        g.run(2)
        out.append((b.split_state(g.get_state()), g.member_stats()))
        g.close()
    (clean, s0), (mixed, s1) = out
    assert [m["status"] for m in s0] == [0, 0, 0]
    assert s1[1]["status"] == 3 and s1[1]["fail_step"] == 1
    for i in (0, 2):
        assert s1[i]["status"] == 0
        for a, ref in zip(mixed[i], clean[i]):
            assert np.array_equal(a, ref)


@pytest.mark.gpu
def test_server_forms_batches(cuda_ok):
    reqs = make_requests(n=8, rate=200.0, seed=9, meshes=((40, 20),), degrees=(2,),
                         steps_range=(2, 5))
    srv = Server(batch_size=4)
    res = srv.run(reqs)
    s = summarize(res, srv.makespan)
    assert s["completed"] == 8, s
    assert max(srv.batches) > 1 and sum(srv.batches) == 8


class _FakeServer(Server):
    """Scheduler under test with the device work replaced by a short sleep."""

    def __init__(self, **kw):
        super().__init__(**kw)
        self.groups = []
        self.max_seen = 0

    def _finish(self, reqs, t0, nbytes):
        import time as _t

        from atmospheric_flows_gb300.serving import MemberResult

        with self._lock:
            self.max_seen = max(self.max_seen, self._running)
        _t.sleep(0.02)
        now = _t.perf_counter() - t0
        with self._lock:
            self._in_use -= nbytes
            self._running -= 1
            for r in reqs:
                self.results.append(MemberResult(r.request_id, r.arrival, now, now, r.steps, 1,
                                                 "ok"))
            self._lock.notify_all()

    def _run_member(self, req, t0, nbytes):
        self.groups.append([req.request_id])
        self._finish([req], t0, nbytes)

    def _run_batch(self, reqs, t0, nbytes):
        self.groups.append([r.request_id for r in reqs])
        self._finish(reqs, t0, nbytes)


def test_scheduler_budget_batching_and_limits():
    small = dict(meshes=((40, 20),), degrees=(2,))
    reqs = make_requests(n=20, rate=1e6, seed=4, **small)  # all arrive at once
    big = MemberRequest(99, 0.0, HillParams(nx=320, nz=160, degree=5), 10)
    budget = 6 * member_bytes(reqs[0].params)
    srv = _FakeServer(hbm_budget=budget, max_running=3, batch_size=4)
    res = srv.run(reqs + [big])
    by_id = {r.request_id: r for r in res}
    assert by_id[99].status.startswith("rejected")
    assert all(by_id[r.request_id].status == "ok" for r in reqs)
    # same key: groups of up to 4, never more than 3 contexts at once, budget kept
    assert max(len(g) for g in srv.groups) == 4
    assert sorted(i for g in srv.groups for i in g) == sorted(r.request_id for r in reqs)
    assert srv.max_seen <= 3 and srv.peak_bytes <= budget


def test_scheduler_does_not_mix_keys():
    a = make_requests(n=6, rate=1e6, seed=5, meshes=((40, 20),), degrees=(2,))
    b = make_requests(n=6, rate=1e6, seed=6, meshes=((40, 20),), degrees=(3,))
    for i, r in enumerate(b):
        r.request_id = 100 + i
    srv = _FakeServer(batch_size=8)
    srv.run(a + b)
    for g in srv.groups:
        assert all(i < 100 for i in g) or all(i >= 100 for i in g)


def test_scheduler_batches_small_members_only():
    """A member larger than batch_max_cells runs alone: it fills the GPU by
    itself, and batched it would make its co-residents run its iterations."""
    small = make_requests(n=6, rate=1e6, seed=7, meshes=((40, 20),), degrees=(3,))
    large = make_requests(n=4, rate=1e6, seed=8, meshes=((160, 80),), degrees=(3,))
    for i, r in enumerate(large):
        r.request_id = 100 + i
    srv = _FakeServer(batch_size=4)
    srv.run(small + large)
    assert max(len(g) for g in srv.groups) > 1
    for g in srv.groups:
        assert len(g) == 1 or all(i < 100 for i in g)


@pytest.mark.gpu
def test_batched_mix_of_degrees_and_meshes_completes(cuda_ok):
    """Members of every degree 2-5 on meshes up to 160x80 (those up to 80x40
    batched) served at once from concurrent host threads: every member
    completes.  Members of one degree
    launch the same kernels with block shapes of their own (the autotuner
    tunes per mesh size); a kernel's shared-memory limit is raised once to
    the device maximum, never set per launch, so one thread cannot lower it
    under another's launch."""
    reqs = make_requests(n=24, rate=1e6, seed=11, meshes=((40, 20), (80, 40), (160, 80)),
                         degrees=(2, 3, 4, 5), steps_range=(3, 6))
    srv = Server(batch_size=4, max_running=16)
    res = srv.run(reqs)
    s = summarize(res, srv.makespan)
    assert s["completed"] == 24 and not s["failed"], s
    assert max(srv.batches) > 1
