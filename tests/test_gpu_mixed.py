"""FP32 PDHG with FP64 iterative refinement: the FP64 KKT of the original LP
meets the requested tolerance and the objectives agree with the FP64 oracle
(the objective bar: 1e-6 relative at tight tolerance)."""
import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol
from test_gpu_solve import _infeasible_primal, _unbounded, docs_problem, params

pytestmark = pytest.mark.gpu
FP32 = cp.PRECISION_FP32_REFINE


@pytest.mark.parametrize("eps", [1e-4, 1e-6])
def test_docs_example_mixed(oracle, eps):
    out = cp.solve(docs_problem(), params(oracle, eps=eps), precision=FP32)
    r = out.result
    assert r["status"] == "OPTIMAL"
    assert r["relative_primal_residual"] < eps and r["relative_dual_residual"] < eps
    assert abs(r["primal_objective_value"] - 3.0) <= 40 * eps
    assert out.info["precision"] == FP32


@pytest.mark.parametrize("eps", [1e-4, 1e-6])
def test_random_lp_mixed_matches_fp64_oracle(oracle, eps):
    prob = cp.Problem.generated("random", 2000, 5000, 20000, 0)
    p = params(oracle, eps=eps)
    g = cp.solve(prob, p, precision=FP32).result
    o, _ = ol.oracle_solve(oracle, prob, params(oracle, eps=1e-8))
    assert g["status"] == "OPTIMAL"
    # the FP64 KKT reported for the returned point meets eps ...
    assert g["relative_primal_residual"] < eps and g["relative_dual_residual"] < eps
    assert g["relative_objective_gap"] < eps
    # ... and the objective is within eps of the FP64 oracle's at 1e-8
    assert abs(g["primal_objective_value"] - o["primal_objective_value"]) <= \
        4 * eps * (1 + abs(o["primal_objective_value"]))


def test_mixed_kkt_is_recomputable_on_host(oracle):
    """The returned point's primal residual, recomputed from the original
    data in numpy, matches the reported one."""
    prob = cp.Problem.generated("random", 800, 2000, 8000, 5)
    a = prob.arrays()
    r = cp.solve(prob, params(oracle, eps=1e-6), precision=FP32).result
    import scipy.sparse as sp
    A = sp.csr_matrix((a["vals"], a["col_ind"], a["row_ptr"]), shape=(a["m"], a["n"]))
    ax = A @ r["x"]
    res = ax - np.clip(ax, a["lc"], a["uc"])
    fin = lambda v: np.where(np.isfinite(v), v, 0.0)
    bn = np.sqrt(np.sum(fin(a["lc"])[(a["lc"] != a["uc"])] ** 2) + np.sum(fin(a["uc"]) ** 2))
    rel_p = np.linalg.norm(res) / (1 + bn)
    assert abs(rel_p - r["relative_primal_residual"]) <= 1e-9 + 1e-6 * rel_p
    assert np.all(r["x"] >= a["lv"] - 1e-12) and np.all(r["x"] <= a["uv"] + 1e-12)


@pytest.mark.parametrize("eps", [1e-6, 1e-8])
def test_transport_mixed_tight(oracle, eps):
    """Refinement rounds take the FP32 solve below its precision floor."""
    prob = cp.Problem.generated("transport", 40, 60, 2)
    p = params(oracle, eps=eps)
    out = cp.solve(prob, p, precision=FP32)
    g = out.result
    assert g["relative_primal_residual"] < eps and g["relative_dual_residual"] < eps
    o, _ = ol.oracle_solve(oracle, prob, params(oracle, eps=1e-8))
    assert g["status"] == "OPTIMAL"
    assert abs(g["primal_objective_value"] - o["primal_objective_value"]) <= \
        1e-5 * (1 + abs(o["primal_objective_value"]))


@pytest.mark.parametrize("maker,expect", [(_infeasible_primal, "PRIMAL_INFEASIBLE"),
                                          (_unbounded, "DUAL_INFEASIBLE")])
def test_mixed_infeasibility(oracle, maker, expect):
    g = cp.solve(maker(), params(oracle, iteration_limit=20000), precision=FP32).result
    assert g["status"] == expect
