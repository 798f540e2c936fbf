"""Feasibility polishing (reference src/pdlp_core_op.cu:861-1360) on the GPU
against the oracle's restatement: after an eps 1e-4 solve, PDHG on the primal
and the dual feasibility problems brings each relative residual below the
polishing tolerance; the solve keeps its termination reason and iteration
count, reports the polishing iterations, and the objectives follow the
polished points."""
import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol

pytestmark = pytest.mark.gpu


def _params(oracle, polish=True, eps=1e-4, eps_polish=1e-6):
    p = ol.oracle_params(oracle)
    p.termination_criteria.eps_optimal_relative = eps
    p.termination_criteria.eps_feasible_relative = eps
    p.termination_criteria.eps_feas_polish_relative = eps_polish
    p.feasibility_polishing = polish
    return p


@pytest.mark.parametrize("args", [(300, 800, 3000, 11), (1000, 2500, 10000, 5)])
def test_polishing_matches_oracle(oracle, args):
    prob = cp.Problem.generated("random", *args)
    p = _params(oracle)
    g = cp.solve(prob, p).result
    o, _ = ol.oracle_solve(oracle, prob, p)
    assert g["status"] == o["status"] == "OPTIMAL"
    assert g["total_count"] == o["total_count"]
    # both halves reach the polishing tolerance
    assert g["relative_primal_residual"] <= 1e-6 and o["relative_primal_residual"] <= 1e-6
    assert g["relative_dual_residual"] <= 1e-6
    assert g["feasibility_polishing_time"] > 0
    # the polish loops follow the oracle's schedule (restart decisions may
    # move by an evaluation with rounding)
    assert abs(g["feasibility_iteration"] - o["feasibility_iteration"]) <= \
        0.1 * o["feasibility_iteration"] + 20
    for k in ("primal_objective_value", "dual_objective_value"):
        assert abs(g[k] - o[k]) <= 1e-6 * (1 + abs(o[k])), k
    # the polished point is feasible to the polishing tolerance on the host too
    a = prob.arrays()
    rp, cj, v = a["row_ptr"], a["col_ind"], a["vals"]
    ax = np.zeros(a["m"])
    np.add.at(ax, np.repeat(np.arange(a["m"]), np.diff(rp)), v * g["x"][cj])
    viol = np.maximum(a["lc"] - ax, 0) + np.maximum(ax - a["uc"], 0)
    bn = np.sqrt(np.sum(np.where(np.isfinite(a["lc"]) & (a["lc"] != a["uc"]), a["lc"], 0) ** 2)
                 + np.sum(np.where(np.isfinite(a["uc"]), a["uc"], 0) ** 2))
    assert np.linalg.norm(viol) / (1 + bn) <= 2e-6


def test_polishing_skipped_when_already_feasible(oracle):
    prob = cp.Problem.generated("random", 300, 800, 3000, 11)
    plain = cp.solve(prob, _params(oracle, polish=False)).result
    g = cp.solve(prob, _params(oracle, polish=True, eps_polish=1e-2)).result
    assert g["feasibility_iteration"] == 0 and g["feasibility_polishing_time"] == 0.0
    assert np.array_equal(g["x"], plain["x"]) and np.array_equal(g["y"], plain["y"])


def test_polishing_not_run_on_infeasible(oracle):
    from test_gpu_solve import _infeasible_primal
    p = _params(oracle)
    g = cp.solve(_infeasible_primal(), p).result
    assert g["status"] == "PRIMAL_INFEASIBLE"
    assert g["feasibility_iteration"] == 0
