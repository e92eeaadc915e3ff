"""Continuous-batching server: every request's result is the same served in
a mix (2D batched with other shots, 3D on a side stream overlapping the 2D
epochs, admission gated by the HBM budget) as run alone."""
import numpy as np
import pytest

import simwave_gb300 as sw
from _cases import random_problem, rel_l2

pytestmark = pytest.mark.gpu


def _requests(seed=1, count=10):
    from simwave_gb300.serve import Request
    rng = np.random.default_rng(seed)
    reqs, arrival = [], 0.0
    for i in range(count):
        dim = 3 if rng.random() < 0.3 else 2
        order = int(rng.choice([4, 8, 12, 16]))
        vd = bool(rng.integers(0, 2))
        if dim == 2:
            shape = tuple(int(v) for v in rng.integers(60, 200, size=2))
        else:
            shape = tuple(int(v) for v in rng.integers(24, 40, size=3))
            if vd:
                shape = (shape[0], shape[1], shape[1])
        kw = random_problem(sw, dim, order, vd, "none", int(rng.integers(0, 3)),
                            shape=shape, tf=float(rng.uniform(0.03, 0.08)),
                            seed=seed * 100 + i, nrec=int(rng.integers(2, 9)))
        arrival += float(rng.exponential(1 / 200.0))
        reqs.append(Request(kw, arrival, tag=i))
    return reqs


def _alone(kw):
    from simwave_gb300.device import DeviceProblem
    dp = DeviceProblem(kw)
    dp.run()
    dp.status()
    return dp.u_full_numpy(), dp.shot_record_numpy()


def test_served_results_equal_alone():
    from simwave_gb300.serve import ShotServer, latency_summary
    reqs = _requests()
    server = ShotServer(epoch_steps=16)
    server.serve(reqs, timeout=300)
    server.close()
    for r in reqs:
        u, rec = _alone(r.kwargs)
        assert not r.evicted
        assert rel_l2(r.problem.u_full_numpy(), u) <= 1e-5, r.tag
        assert rel_l2(r.shot_record, rec) <= 1e-5, r.tag
    s = latency_summary(reqs)
    assert s["shots"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0


def test_budget_gates_admission():
    from simwave_gb300.serve import ShotServer
    reqs = _requests(seed=4, count=6)
    budget = max(r.bytes for r in reqs) + 1
    server = ShotServer(hbm_budget=budget, epoch_steps=8)
    peak = []
    orig = server._admit

    def admit(now):
        out = orig(now)
        peak.append(server.in_use - server.resident)
        return out

    server._admit = admit
    server.serve(reqs, timeout=300)
    server.close()
    assert all(r.completed is not None for r in reqs)
    assert max(peak) <= budget


def test_stream_shots_run_shortest_first():
    """Side-stream shots admitted together complete in order of size."""
    from simwave_gb300.serve import Request, ShotServer
    reqs = []
    for i, n in enumerate((40, 24, 32, 28)):
        kw = random_problem(sw, 3, 4, False, "none", 0, shape=(n, n, n), tf=0.05,
                            seed=70 + i, nrec=3)
        reqs.append(Request(kw, 0.0, tag=i))
    server = ShotServer(inflight=1)
    server.prepare(reqs)  # all staged: the order is the server's choice alone
    server.serve(reqs, timeout=300)
    server.close()
    order = [r.tag for r in sorted(reqs, key=lambda r: r.completed)]
    assert order == [r.tag for r in sorted(reqs, key=lambda r: r.updates)]


def test_3d_shots_overlap_2d_epochs_and_each_other():
    """3D shots run while the 2D batch is stepping and several at once, and
    every result equals the shot run alone."""
    from simwave_gb300.serve import Request, ShotServer
    reqs = []
    for i in range(4):  # 2D shots long enough to keep the batch busy
        kw = random_problem(sw, 2, 8, bool(i % 2), "none", 0, shape=(300, 420),
                            tf=0.4, seed=200 + i, nrec=6)
        reqs.append(Request(kw, 0.0, tag="2d%d" % i))
    for i in range(3):
        kw = random_problem(sw, 3, 8, i == 1, "none", 0, shape=(40, 44, 44),
                            tf=0.08, seed=300 + i, nrec=5)
        reqs.append(Request(kw, 0.0, tag="3d%d" % i))
    server = ShotServer(epoch_steps=16, inflight=3, inflight_beside_2d=3)
    server.prepare(reqs)
    server.serve(reqs, timeout=300)
    server.close()
    two = [r for r in reqs if r.kind == "2d"]
    three = [r for r in reqs if r.kind == "3d"]
    last2d = max(r.completed for r in two)
    assert any(r.started < last2d for r in three), "no 3D shot ran beside the 2D batch"
    assert any(a.started < b.completed and b.started < a.completed
               for a in three for b in three if a is not b), "3D shots ran one at a time"
    for r in reqs:
        u, rec = _alone(r.kwargs)
        assert rel_l2(r.problem.u_full_numpy(), u) <= 1e-5, r.tag
        assert rel_l2(r.shot_record, rec) <= 1e-5, r.tag
