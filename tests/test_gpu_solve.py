"""End-to-end parity of the GPU solve with the CPU oracle (same seeded LPs,
same parameters), through the reference-compatible C API."""
import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol

pytestmark = pytest.mark.gpu


def params(oracle, **kw):
    p = ol.oracle_params(oracle)
    for k, v in kw.items():
        if k in ("eps", "eps_opt", "eps_feas"):
            if k in ("eps", "eps_opt"):
                p.termination_criteria.eps_optimal_relative = v
            if k in ("eps", "eps_feas"):
                p.termination_criteria.eps_feasible_relative = v
        elif k == "iteration_limit":
            p.termination_criteria.iteration_limit = v
        else:
            setattr(p, k, v)
    return p


def docs_problem():
    # reference docs/C_API.md:47-90: min x1 + x2, x1 + 2 x2 = 5, x2 <= 2,
    # 3 x1 + 2 x2 <= 8, x free -> x = (1, 2), objective 3
    return cp.Problem.from_csr([0, 2, 3, 5], [0, 1, 1, 0, 1], [1.0, 2.0, 1.0, 3.0, 2.0], 2,
                               c=[1.0, 1.0], lc=[5.0, -np.inf, -np.inf], uc=[5.0, 2.0, 8.0])


def test_docs_example_known_answer(oracle):
    prob = docs_problem()
    for eps in (1e-4, 1e-8):
        out = cp.solve(prob, params(oracle, eps=eps))
        r = out.result
        assert r["status"] == "OPTIMAL"
        assert abs(r["primal_objective_value"] - 3.0) <= 10 * eps * 4
        np.testing.assert_allclose(r["x"], [1.0, 2.0], atol=50 * eps)
        o, _ = ol.oracle_solve(oracle, prob, params(oracle, eps=eps))
        assert abs(r["total_count"] - o["total_count"]) <= 20


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_random_lp_trace_and_objective_match_oracle(oracle, seed):
    prob = cp.Problem.generated("random", 2000, 5000, 20000, seed)
    p = params(oracle, eps=1e-4)
    g = cp.solve(prob, p, trace_cap=4000)
    o, otr = ol.oracle_solve(oracle, prob, p, trace_cap=4000)
    gr = g.result
    assert gr["status"] == o["status"] == "OPTIMAL"
    # same evaluation schedule: identical iteration stamps on the common prefix
    k = min(len(g.trace), len(otr))
    assert k >= 5
    np.testing.assert_array_equal(g.trace[:k, 0], otr[:k, 0])
    # the first evaluations agree to rounding (1e-9 relative on the first 20)
    early = min(k, 20)
    for col in (1, 2, 3, 6):
        np.testing.assert_allclose(g.trace[:early, col], otr[:early, col], rtol=1e-8, atol=1e-12)
    # iteration count to 1e-4 within 2% of the oracle's, objectives to 1e-6,
    # result vectors (x, y, reduced cost) to 1e-7 of their largest entry
    assert abs(gr["total_count"] - o["total_count"]) <= 0.02 * o["total_count"] + 10
    for key in ("primal_objective_value", "dual_objective_value"):
        assert abs(gr[key] - o[key]) <= 1e-6 * (1 + abs(o[key]))
    for key in ("x", "y", "rc"):
        assert np.max(np.abs(gr[key] - o[key])) <= 1e-7 * (1 + np.max(np.abs(o[key])))


def test_tight_tolerance_objectives_agree(oracle):
    prob = cp.Problem.generated("random", 300, 700, 3000, 9)
    p = params(oracle, eps=1e-8)
    g = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert g["status"] == o["status"] == "OPTIMAL"
    for key in ("primal_objective_value", "dual_objective_value"):
        assert abs(g[key] - o[key]) <= 1e-6 * (1 + abs(o[key]))
    # own KKT of the returned (unscaled) solution meets eps
    assert g["relative_primal_residual"] < 1e-8 and g["relative_dual_residual"] < 1e-8


def test_linf_norm_and_no_rescaling(oracle):
    prob = cp.Problem.generated("random", 400, 900, 4000, 4)
    p = params(oracle, eps=1e-6, optimality_norm=cp.NORM_LINF, l_inf_ruiz_iterations=0,
               has_pock_chambolle_alpha=False, bound_objective_rescaling=False)
    g = cp.solve(prob, p, trace_cap=2000)
    o, otr = ol.oracle_solve(oracle, prob, p, trace_cap=2000)
    assert g.result["status"] == o["status"]
    k = min(len(g.trace), len(otr), 10)
    np.testing.assert_allclose(g.trace[:k, 1:4], otr[:k, 1:4], rtol=1e-8, atol=1e-13)
    assert abs(g.result["primal_objective_value"] - o["primal_objective_value"]) <= \
        1e-5 * (1 + abs(o["primal_objective_value"]))


def test_iteration_limit(oracle):
    prob = cp.Problem.generated("random", 500, 1200, 6000, 3)
    p = params(oracle, eps=1e-12, iteration_limit=333)
    g = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert g["status"] == o["status"] == "ITERATION_LIMIT"
    assert g["total_count"] == o["total_count"] == 333
    np.testing.assert_allclose(g["relative_primal_residual"], o["relative_primal_residual"],
                               rtol=1e-6)


def _infeasible_primal():
    # x1 + x2 <= 1 and x1 + x2 >= 3, x >= 0
    return cp.Problem.from_csr([0, 2, 4], [0, 1, 0, 1], [1.0, 1.0, 1.0, 1.0], 2,
                               c=[1.0, 1.0], lc=[-np.inf, 3.0], uc=[1.0, np.inf],
                               lv=[0.0, 0.0], uv=[np.inf, np.inf])


def _unbounded():
    # min -x1 s.t. x1 - x2 >= 0, x >= 0   (ray x1 = x2 -> -inf)
    return cp.Problem.from_csr([0, 2], [0, 1], [1.0, -1.0], 2, c=[-1.0, 0.0], lc=[0.0],
                               uc=[np.inf], lv=[0.0, 0.0], uv=[np.inf, np.inf])


@pytest.mark.parametrize("maker,expect", [(_infeasible_primal, "PRIMAL_INFEASIBLE"),
                                          (_unbounded, "DUAL_INFEASIBLE")])
def test_infeasibility_detection_matches_oracle(oracle, maker, expect):
    prob = maker()
    p = params(oracle, iteration_limit=20000)
    g = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert o["status"] == expect
    assert g["status"] == expect
    assert g["total_count"] == o["total_count"]


def test_warm_start_from_solution_converges_fast(oracle):
    prob = cp.Problem.generated("random", 1000, 2500, 10000, 21)
    p = params(oracle, eps=1e-6)
    cold = cp.solve(prob, p).result
    prob.set_start(cold["x"], cold["y"])
    warm = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert warm["status"] == "OPTIMAL"
    assert warm["total_count"] < cold["total_count"]
    assert abs(warm["total_count"] - o["total_count"]) <= 0.1 * o["total_count"] + 20


def test_empty_rows_columns_and_free_variables(oracle):
    # row 1 empty (0 <= 0 <= 5), column 2 empty with a free bound and zero cost
    prob = cp.Problem.from_csr([0, 2, 2, 4], [0, 1, 0, 1], [1.0, 1.0, 1.0, -1.0], 3,
                               c=[1.0, 2.0, 0.0], lc=[1.0, 0.0, -1.0], uc=[4.0, 5.0, 1.0],
                               lv=[0.0, 0.0, -np.inf], uv=[np.inf, np.inf, np.inf])
    p = params(oracle, eps=1e-8)
    g = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert g["status"] == o["status"] == "OPTIMAL"
    assert abs(g["primal_objective_value"] - 1.0) < 1e-6
    assert abs(g["total_count"] - o["total_count"]) <= 20


def test_invalid_csr_returns_null_not_fault(lib):
    # column index out of range: the C API must refuse, not touch the GPU out of bounds
    prob = cp.Problem.from_csr([0, 2], [0, 7], [1.0, 1.0], 2, c=[1.0, 1.0], lc=[1.0],
                               uc=[1.0], lv=[0.0, 0.0], uv=[1.0, 1.0])
    r = lib.solve_lp_problem(prob.ptr, None)
    assert not r
    assert b"invalid CSR" in lib.pdlp_last_error()


def test_null_problem_returns_null(lib):
    assert not lib.solve_lp_problem(None, None)


def test_repeat_solve_is_bitwise_reproducible(oracle):
    prob = cp.Problem.generated("random", 900, 2000, 9000, 13)
    p = params(oracle)
    a = cp.solve(prob, p).result
    b = cp.solve(prob, p).result
    assert a["total_count"] == b["total_count"]
    assert np.array_equal(a["x"], b["x"]) and np.array_equal(a["y"], b["y"])


def test_in_loop_kernel_timing_is_reported(lib):
    """Events captured into the chunk graphs time one ordinary primal and dual
    launch per 100-iteration chunk; the averages agree with isolated launches."""
    prob = cp.Problem.generated("random", 2000, 5000, 20000, 0)
    params = cp.default_parameters()
    params.presolve = False
    dp = cp.DeviceProblem(prob)
    try:
        out = dp.solve(params)
        info = out.info
        assert out.result["status"] == "OPTIMAL"
        assert info["timed_chunks"] >= out.result["total_count"] // 100 - 3
        ms = dp.time_kernels(params, reps=10)
        for live, iso in ((info["primal_step_ms"], ms[0]), (info["dual_step_ms"], ms[1])):
            assert 0 < live < 5 * iso + 0.05, (live, iso)
        # the sampled events leave the solve unchanged
        again = dp.solve(params).result
        assert again["total_count"] == out.result["total_count"]
        assert np.array_equal(again["x"], out.result["x"])
    finally:
        dp.free()
