"""The command-line tool end to end: MPS in, the reference's three output
files out, with the optimum of the problem."""
import os
import subprocess

import numpy as np
import pytest

import cupdlpx as cp

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _run(args, tmp_path):
    cli = os.path.join(os.path.dirname(cp.LIB_PATH), "cupdlpx")
    env = dict(os.environ, PDLP_QUIET="1")
    return subprocess.run([cli] + args + [os.path.join(HERE, "golden", "mps", "basic.mps"),
                                          str(tmp_path)], capture_output=True, text=True, env=env)


def _summary(tmp_path):
    out = {}
    for line in open(tmp_path / "basic_summary.txt"):
        k, v = line.split(":", 1)
        out[k.strip()] = v.strip()
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cli_writes_summary_and_solutions(tmp_path, precision):
    r = _run(["--eps_opt", "1e-7", "--eps_feas", "1e-7", "--no_presolve", "--precision",
              precision], tmp_path)
    assert r.returncode == 0, r.stderr
    s = _summary(tmp_path)
    assert s["Termination Reason"] == "OPTIMAL"
    assert s["Rows"] == "3" and s["Columns"] == "3" and s["Nonzeros"] == "6"
    # min x1 + 2 x2 - x3 s.t. x1 + x2 <= 4, x2 + x3 >= 1, x1 - x3 = 0.5,
    # 0 <= x1 <= 3, x2 >= 0.5, x3 free: optimum 1.5 (x2 = 0.5, a segment of x1)
    assert abs(float(s["Primal Objective Value"]) - 1.5) < 1e-5
    x = np.loadtxt(tmp_path / "basic_primal_solution.txt")
    y = np.loadtxt(tmp_path / "basic_dual_solution.txt")
    assert x.shape == (3,) and y.shape == (3,)
    tol = 1e-5
    assert abs(x[0] - x[2] - 0.5) < tol and x[0] + x[1] <= 4 + tol and x[1] + x[2] >= 1 - tol
    assert -tol <= x[0] <= 3 + tol and x[1] >= 0.5 - tol


def test_cli_missing_file_fails(tmp_path):
    cli = os.path.join(os.path.dirname(cp.LIB_PATH), "cupdlpx")
    r = subprocess.run([cli, str(tmp_path / "absent.mps"), str(tmp_path)], capture_output=True,
                       text=True)
    assert r.returncode == 1
