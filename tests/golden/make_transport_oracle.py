"""Write tests/golden/transport_20m_1e8.json: the FP64 oracle of the
configured mixed-precision LP.

The LP is the seeded transportation problem (2,000 sources x 5,000 sinks:
n = 10M arcs, m = 7,000 rows, nnz = 20M, seed 2).  Its FP64 oracle is the
reference's own single-GPU FP64 solve (src/solver.cu optimize() through
solve_lp_problem, built by `make -C oracle refgpu`) run to relative KKT
1e-8; this library's FP64 solve to 1e-8 is recorded beside it.  The
fixture keeps the scalars only (objectives, residuals, iterations), so the
GPU tests can check an FP32 + refinement solve against the oracle in
seconds instead of the minutes the 1e-8 solves take.

Run on a machine with a GPU and the staged reference build:
    python tests/golden/make_transport_oracle.py [output.json]
"""
from __future__ import annotations

import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "d-pdlp_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import cupdlpx as cp  # noqa: E402
import oracle_lib as ol  # noqa: E402

OUT = os.path.join(HERE, "transport_20m_1e8.json")
KEYS = ("status", "total_count", "primal_objective_value", "dual_objective_value",
        "relative_primal_residual", "relative_dual_residual", "relative_objective_gap")


def main(out: str = OUT) -> None:
    prob = cp.Problem.generated("transport", 2000, 5000, 2)
    t0 = time.perf_counter()
    ref = ol.ref_gpu_solve(prob, eps=1e-8, timeout=7200)
    t_ref = time.perf_counter() - t0
    p = ol.oracle_params(ol.load())
    p.termination_criteria.eps_optimal_relative = 1e-8
    p.termination_criteria.eps_feasible_relative = 1e-8
    t0 = time.perf_counter()
    ours = cp.solve(prob, p, precision=cp.PRECISION_FP64).result
    t_ours = time.perf_counter() - t0
    doc = {
        "lp": "transport 2000 x 5000, seed 2 (n = 10,000,000, m = 7,000, nnz = 20,000,000)",
        "eps": 1e-8,
        "reference_fp64": {k: ref[k] for k in KEYS} | {"wall_s": round(ref["wall_s"], 2),
                                                      "process_s": round(t_ref, 2)},
        "ours_fp64": {k: ours[k] for k in KEYS} | {"wall_s": round(t_ours, 2)},
    }
    with open(out, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(doc))


if __name__ == "__main__":
    main(*sys.argv[1:])
