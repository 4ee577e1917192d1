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
