"""Parity at the benchmark sizes: the 20M-nnz power-law LP (m = 1,000,000,
n = 2,000,000) and the 20M-nnz transportation LP (2,000 x 5,000), run for a
few hundred iterations on the GPU and on the oracle from the same seeded
problem.  Both follow the same evaluation schedule; the KKT measures of the
early evaluations agree to rounding, the power-method step size agrees, and
the returned point's KKT recomputed on the host matches the reported one."""
import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol
from test_gpu_solve import params

pytestmark = pytest.mark.gpu

ITERS = 400

FULL = [("powerlaw", (1000000, 2000000, 20000000, 1.2, 50000, 1)),
        ("transport", (2000, 5000, 2))]


def _host_rel_primal(prob, x):
    a = prob.arrays()
    rp, cj, v = a["row_ptr"], a["col_ind"], a["vals"]
    ax = np.bincount(np.repeat(np.arange(a["m"]), np.diff(rp)), weights=v * x[cj],
                     minlength=a["m"])
    viol = np.maximum(a["lc"] - ax, 0.0) + np.maximum(ax - a["uc"], 0.0)
    lc, uc = a["lc"], a["uc"]
    bn2 = np.sum(np.where(np.isfinite(lc) & (lc != uc), lc, 0.0) ** 2) + \
        np.sum(np.where(np.isfinite(uc), uc, 0.0) ** 2)
    return np.linalg.norm(viol) / (1.0 + np.sqrt(bn2))


@pytest.mark.parametrize("kind,args", FULL, ids=["powerlaw_20M", "transport_20M"])
def test_full_size_trace_matches_oracle(oracle, kind, args):
    prob = cp.Problem.generated(kind, *args)
    p = params(oracle, eps=1e-12, iteration_limit=ITERS)
    g = cp.solve(prob, p, trace_cap=200)
    o, otr = ol.oracle_solve(oracle, prob, p, trace_cap=200)
    gr = g.result
    assert gr["status"] == o["status"] == "ITERATION_LIMIT"
    assert gr["total_count"] == o["total_count"] == ITERS
    k = min(len(g.trace), len(otr))
    assert k >= 10
    np.testing.assert_array_equal(g.trace[:k, 0], otr[:k, 0])
    # step size from the power method, and the early KKT measures
    np.testing.assert_allclose(g.trace[0, 8], otr[0, 8], rtol=1e-10)
    early = min(k, 12)
    for col in (1, 2, 3):
        np.testing.assert_allclose(g.trace[:early, col], otr[:early, col], rtol=1e-7, atol=1e-14)
    for key in ("relative_primal_residual", "relative_dual_residual", "relative_objective_gap"):
        np.testing.assert_allclose(gr[key], o[key], rtol=1e-5, atol=1e-12)
    # the reported primal residual is that of the returned point
    np.testing.assert_allclose(_host_rel_primal(prob, gr["x"]), gr["relative_primal_residual"],
                               rtol=1e-6, atol=1e-12)
