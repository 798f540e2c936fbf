"""Batched and served solves (pdlp_batch_solve, pdlp_server_*).

Each LP's arithmetic depends on its own data only, so its result must be
bitwise the same solved alone and in the mix, whatever else is in flight;
admission by memory budget must serialise requests without deadlock.
"""
import threading
import time

import numpy as np
import pytest

import cupdlpx as cp

pytestmark = pytest.mark.gpu


def _params(eps=1e-4):
    p = cp.default_parameters()
    p.presolve = False
    p.termination_criteria.eps_optimal_relative = eps
    p.termination_criteria.eps_feasible_relative = eps
    return p


def _mixed_lps(count, seed0=100):
    rng = np.random.default_rng(seed0)
    lps = []
    for i in range(count):
        m = int(rng.integers(150, 2500))
        n = int(2.5 * m)
        lps.append(cp.Problem.generated("random", m, n, 10 * n, seed0 + i))
    return lps


def _same(a, b):
    assert a["status"] == b["status"]
    assert a["total_count"] == b["total_count"]
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["y"], b["y"])
    assert a["primal_objective_value"] == b["primal_objective_value"]


def test_batch_results_equal_alone():
    lps = _mixed_lps(16)
    p = _params()
    alone = [cp.solve(lp, p).result for lp in lps]
    batch, info = cp.batch_solve(lps, p, workers=8)
    assert info["lps"] == 16 and info["failed"] == 0
    assert info["max_concurrent"] > 1
    for a, b in zip(alone, batch):
        assert a["status"] == "OPTIMAL"
        _same(a, b)


def test_server_staggered_arrivals_equal_alone():
    lps = _mixed_lps(12, seed0=300)
    p = _params()
    alone = [cp.solve(lp, p).result for lp in lps]
    with cp.Server(p, workers=4) as srv:
        ids = []

        def submit():
            for lp in lps:
                ids.append(srv.submit(lp))
                time.sleep(0.002)

        th = threading.Thread(target=submit)
        th.start()
        th.join()
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["completed"] == 12 and st["failed"] == 0
    for a, (b, info) in zip(alone, got):
        _same(a, b)
        assert info["latency_seconds"] >= info["solve_seconds"] > 0
        assert info["device_bytes"] > 0
        # the solve's stream time and the host upload lie inside the request's solve time
        assert 0 < info["device_seconds"] <= info["solve_seconds"] + 1e-3
        assert 0 <= info["upload_seconds"] <= info["solve_seconds"]


def test_memory_budget_serialises_admission():
    lps = _mixed_lps(6, seed0=500)
    p = _params()
    # a budget below any single footprint: one request in flight at a time
    res, info = cp.batch_solve(lps, p, workers=4, mem_budget_bytes=1)
    assert info["failed"] == 0 and info["max_concurrent"] == 1
    for lp, r in zip(lps, res):
        _same(cp.solve(lp, p).result, r)


def test_mixed_precision_batch_equals_alone():
    lps = _mixed_lps(4, seed0=700)
    p = _params(1e-6)
    fp32 = cp.PRECISION_FP32_REFINE
    alone = [cp.solve(lp, p, precision=fp32).result for lp in lps]
    batch, info = cp.batch_solve(lps, p, precision=fp32, workers=4)
    assert info["failed"] == 0
    for a, b in zip(alone, batch):
        assert b["status"] == "OPTIMAL"
        _same(a, b)


def test_failed_request_reports_error_and_others_finish():
    good = _mixed_lps(2, seed0=900)
    bad = cp.Problem.from_csr([0, 2], [0, 7], [1.0, 1.0], 3, c=[1.0, 1.0, 1.0])  # column 7 >= n
    p = _params()
    res, info = cp.batch_solve([good[0], bad, good[1]], p, workers=2)
    assert info["failed"] == 1
    assert res[1] is None and res[0] is not None and res[2] is not None


def test_wire_payloads_solve_like_problems():
    lps = _mixed_lps(3, seed0=950)
    p = _params()
    with cp.Server(p, workers=2) as srv:
        ids = [srv.submit_bytes(lp.to_bytes()) for lp in lps]
        got = [srv.wait(i)[0] for i in ids]
    for lp, g in zip(lps, got):
        _same(cp.solve(lp, p).result, g)


def test_queue_bound_refuses_and_accepted_requests_equal_alone():
    # one worker and a 1-byte bound: a request is queued only when nothing
    # waits, so a burst of submissions is partly refused (-2, counted); every
    # accepted request still completes, bitwise as alone
    lps = _mixed_lps(10, seed0=500)
    p = _params()
    with cp.Server(p, workers=1) as srv:
        srv.set_queue_limit(1)
        ids = [srv.submit(lp) for lp in lps]
        results = {k: srv.wait(rid)[0] for k, rid in enumerate(ids) if rid >= 0}
        st = srv.stats()
    refused = sum(1 for rid in ids if rid == -2)
    assert refused >= 1 and st["rejected"] == refused
    assert len(results) == 10 - refused and st["queued_host_bytes"] == 0
    for k, res in results.items():
        _same(res, cp.solve(lps[k], p).result)
