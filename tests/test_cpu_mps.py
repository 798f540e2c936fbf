"""MPS reader and command-line tool on CPU.

read_mps_file must give the reference reader's problem (src/mps_parser.c) on
every fixture under tests/golden/mps: the fixtures cover section order,
comments, several and missing N rows, OBJSENSE, objective constants, RANGES
of every sign and row type, every bound kind, integer markers, continuation
lines, unknown names, duplicate entries and gzip input.  Golden outputs of
the reference reader are in tests/golden/ref_mps.npz; where the reference
was built here, the check also runs live.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol

HERE = os.path.dirname(os.path.abspath(__file__))
MPS_DIR = os.path.join(HERE, "golden", "mps")
KEYS = ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv")


@pytest.fixture(scope="module")
def golden_mps():
    return np.load(os.path.join(HERE, "golden", "ref_mps.npz"))


def _ours(lib, name):
    return cp.Problem.from_mps(os.path.join(MPS_DIR, name), library=lib).arrays()


def test_fixture_set_is_complete(golden_mps):
    names = sorted(f for f in os.listdir(MPS_DIR) if ".mps" in f)
    assert names == [str(n) for n in golden_mps["names"]]


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(MPS_DIR) if ".mps" in f))
def test_mps_matches_reference_golden(lib, golden_mps, name):
    if name.endswith(".gz") and not os.path.exists("/usr/include/zlib.h"):
        pytest.skip("library built without zlib")
    a = _ours(lib, name)
    assert [a["m"], a["n"], a["nnz"]] == list(golden_mps[f"{name}__shape"])
    for k in KEYS:
        assert np.array_equal(a[k], golden_mps[f"{name}__{k}"]), k
    assert a["c0"] == float(golden_mps[f"{name}__c0"])


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(MPS_DIR) if ".mps" in f))
def test_mps_matches_reference_live(lib, ref, name):
    ref.read_mps_file.restype = C.POINTER(cp.LpProblem)
    ref.read_mps_file.argtypes = [C.c_char_p]
    pp = ref.read_mps_file(os.path.join(MPS_DIR, name).encode())
    b = cp.problem_arrays(pp)
    a = _ours(lib, name)
    for k in KEYS:
        assert np.array_equal(a[k], b[k]), k
    assert a["c0"] == b["c0"]
    ref.lp_problem_free(pp)


def test_missing_mps_file_returns_null(lib, tmp_path):
    assert not lib.read_mps_file(str(tmp_path / "absent.mps").encode())


def test_mps_round_trip_through_oracle(lib, oracle):
    """A parsed file solves to the same optimum as the LP written by hand."""
    prob = cp.Problem.from_mps(os.path.join(MPS_DIR, "basic.mps"), library=lib)
    p = ol.oracle_params(oracle)
    p.termination_criteria.eps_optimal_relative = 1e-8
    p.termination_criteria.eps_feasible_relative = 1e-8
    r, _ = ol.oracle_solve(oracle, prob, p)
    assert r["status"] == "OPTIMAL"
    # min x1 + 2 x2 - x3: x1 + x2 <= 4, x2 + x3 >= 1, x1 - x3 = 0.5,
    # 0 <= x1 <= 3, x2 >= 0.5, x3 <= +inf (lower -inf)
    from scipy.optimize import linprog
    res = linprog([1, 2, -1], A_ub=[[1, 1, 0], [0, -1, -1]], b_ub=[4, -1],
                  A_eq=[[1, 0, -1]], b_eq=[0.5],
                  bounds=[(0, 3), (0.5, None), (None, None)], method="highs")
    assert abs(r["primal_objective_value"] - res.fun) < 1e-6 * (1 + abs(res.fun))


def test_cli_usage_and_argument_errors():
    cli = os.path.join(os.path.dirname(cp.LIB_PATH), "cupdlpx")
    if not os.path.exists(cli):
        pytest.skip("command-line tool not built")
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "<mps_file> <output_dir>" in r.stderr
    r = subprocess.run([cli, "only_one_argument"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([cli, "--opt_norm", "l3", "a.mps", "out"], capture_output=True, text=True)
    assert r.returncode == 1


def test_mutated_mps_files_parse_or_fail_cleanly(lib, tmp_path):
    """Lines deleted, duplicated, truncated or replaced with noise: the reader
    returns a problem or NULL, never crashes, and what it returns is a valid
    CSR problem."""
    import random
    texts = [open(os.path.join(MPS_DIR, f)).read() for f in sorted(os.listdir(MPS_DIR))
             if f.endswith(".mps")]
    rng = random.Random(7)
    path = tmp_path / "m.mps"
    for _ in range(400):
        lines = rng.choice(texts).split("\n")
        for _ in range(rng.randint(1, 5)):
            i = rng.randrange(len(lines))
            op = rng.randint(0, 4)
            if op == 0 and len(lines) > 1:
                del lines[i]
            elif op == 1:
                lines.insert(i, rng.choice(lines))
            elif op == 2:
                lines[i] = lines[i][: rng.randrange(len(lines[i]) + 1)]
            elif op == 3:
                lines[i] += " " + rng.choice(["1e400", "-inf", "nan", "X", "9" * 30, "MARKER"])
            else:
                lines[i] = "".join(rng.choice("AB 01.-+eE\t") for _ in range(rng.randint(0, 30)))
        path.write_text("\n".join(lines))
        p = lib.read_mps_file(os.fsencode(str(path)))
        if p:
            a = cp.problem_arrays(p)
            rp = a["row_ptr"]
            assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and rp[-1] == a["nnz"]
            assert np.all((a["col_ind"] >= 0) & (a["col_ind"] < a["n"]))
            lib.lp_problem_free(p)
