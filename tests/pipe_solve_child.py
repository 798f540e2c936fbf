"""Child process of tests/test_gpu_pipe.py: solves seeded LPs with the SpMV
kernel forced by PDLP_STEP_KERNEL (read once per process) and prints the
results as one JSON line."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "d-pdlp_gb300"))
sys.path.insert(0, HERE)

import cupdlpx as cp  # noqa: E402
import oracle_lib as ol  # noqa: E402

LPS = {
    # A: rows of ~20 (packed tiles); A^T: columns of Zipf degrees up to
    # 5,000 (one-row tiles, chunks of long rows)
    "powerlaw": ("powerlaw", 20000, 40000, 400000, 1.2, 5000, 3),
    # rows of 200 and 50: one-row and packed tiles
    "transport": ("transport", 50, 200, 4),
    "random": ("random", 2000, 5000, 20000, 0),
}


def main():
    eps = float(sys.argv[1])
    out = {}
    for name, args in LPS.items():
        prob = cp.Problem.generated(*args)
        p = ol.oracle_params(ol.load())
        p.termination_criteria.eps_optimal_relative = eps
        p.termination_criteria.eps_feasible_relative = eps
        for prec_name, prec in (("fp64", cp.PRECISION_FP64), ("fp32", cp.PRECISION_FP32_REFINE)):
            o = cp.solve(prob, p, precision=prec)
            r = o.result
            out[f"{name}/{prec_name}"] = {
                k: r[k] for k in ("status", "total_count", "primal_objective_value",
                                  "dual_objective_value", "relative_primal_residual",
                                  "relative_dual_residual", "relative_objective_gap")
            } | {"kernel_A": o.info.get("spmv_kernel_A"), "kernel_AT": o.info.get("spmv_kernel_AT")}
    print("PIPE_RESULT " + json.dumps(out))


if __name__ == "__main__":
    main()
