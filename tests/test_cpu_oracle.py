"""The oracle pinned against the reference (CPU only).

Golden file tests/golden/ref_host.npz holds outputs of the reference's own
host code (written by tests/golden/make_golden.py).  The oracle must match
it bit for bit on:
  - rescaling (reference src/preconditioner.c:89-273);
  - the dense / CSC / COO converters of create_lp_problem
    (reference src/utils.cu:816-1013);
  - default parameters (src/utils.cu:295-329);
  - the evaluation cadence (src/utils.cu:492-501);
  - the termination and restart decisions (src/utils.cu:214-293).
Where the reference was built here (oracle/_ref), the same checks also run
live against it.

The reference's iteration loop is CUDA and cannot run on a CPU host.  It is
pinned through the documented example's known answer and through agreement
with SciPy's HiGHS on seeded LPs.
"""
import ctypes as C
import os

import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_host.npz")
RESCALE_KEYS = ("vals", "c", "lv", "uv", "lc", "uc", "con", "var")
N_LPS = 4
N_CONV = 6


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def _golden_problem(g, i, library):
    return cp.Problem.from_csr(g[f"lp{i}_row_ptr"], g[f"lp{i}_col_ind"], g[f"lp{i}_vals"],
                               int(g[f"lp{i}_n"]), c=g[f"lp{i}_c"], lc=g[f"lp{i}_lc"],
                               uc=g[f"lp{i}_uc"], lv=g[f"lp{i}_lv"], uv=g[f"lp{i}_uv"],
                               library=library)


def _rescale_params(O, row):
    p = ol.oracle_params(O)
    p.l_inf_ruiz_iterations = int(row[0])
    p.has_pock_chambolle_alpha = bool(row[1])
    p.pock_chambolle_alpha = float(row[2])
    p.bound_objective_rescaling = bool(row[3])
    return p


def _bind_decisions(lib):
    lib.oracle_termination_decision.restype = C.c_int
    lib.oracle_termination_decision.argtypes = [C.POINTER(cp.TerminationCriteria)] + [
        C.c_double] * 7 + [C.c_int, C.c_double]
    lib.oracle_restart_decision.restype = C.c_int
    lib.oracle_restart_decision.argtypes = [C.POINTER(cp.RestartParameters), C.c_int, C.c_int,
                                            C.c_int, C.c_double, C.c_double, cp._dp]


@pytest.mark.parametrize("i", range(N_LPS))
def test_rescaling_matches_reference_golden(lib, oracle, golden, i):
    prob = _golden_problem(golden, i, lib)
    for j, row in enumerate(golden["rescale_sets"]):
        out = ol.oracle_rescale(oracle, prob, _rescale_params(oracle, row))
        for k in RESCALE_KEYS:
            assert np.array_equal(out[k], golden[f"resc{i}_{j}_{k}"]), (i, j, k)
        assert [out["cb"], out["ob"]] == list(golden[f"resc{i}_{j}_cbob"]), (i, j)


@pytest.mark.parametrize("i", range(N_LPS))
def test_rescaling_matches_reference_live(lib, oracle, ref, golden, i):
    prob = _golden_problem(golden, i, lib)
    for row in golden["rescale_sets"]:
        p = _rescale_params(oracle, row)
        a, b = ol.oracle_rescale(oracle, prob, p), ol.ref_rescale(ref, prob, p)
        for k in RESCALE_KEYS:
            assert np.array_equal(a[k], b[k]), k
        assert (a["cb"], a["ob"]) == (b["cb"], b["ob"])


def test_generators_reproduce_golden_inputs(lib, golden):
    """The seeded generators give the stored LPs bit for bit on this host."""
    import make_golden
    for i, (kind, args) in enumerate(make_golden.LPS):
        a = cp.Problem.generated(kind, *args, library=lib).arrays()
        for k in ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv"):
            assert np.array_equal(a[k], golden[f"lp{i}_{k}"]), (i, k)


def _converter_descs():
    import make_golden
    return [make_golden.desc_for(kind, tol, data)
            for kind, tol, data in make_golden.converter_cases()]


def test_converters_match_reference(lib, oracle, golden):
    descs = _converter_descs()
    assert len(descs) == N_CONV
    for i, (d, _keep) in enumerate(descs):
        want = [golden[f"conv{i}_{k}"] for k in ("row_ptr", "col_ind", "vals")]
        # the product's create_lp_problem (host code of the library)
        c = np.zeros(d.n)
        pp = lib.create_lp_problem(cp.as_dp(c), C.byref(d), None, None, None, None, None)
        assert pp
        a = cp.problem_arrays(pp)
        got = [a["row_ptr"], a["col_ind"], a["vals"]]
        for k, w, x in zip(("row_ptr", "col_ind", "vals"), want, got):
            assert np.array_equal(w, x), (i, k)
        for k in ("lc", "uc", "lv", "uv"):
            assert np.array_equal(a[k], golden[f"conv{i}_{k}"]), (i, k)
        lib.lp_problem_free(pp)
        # the oracle's converters
        fn = {cp.MATRIX_DENSE: oracle.oracle_dense_to_csr, cp.MATRIX_CSC: oracle.oracle_csc_to_csr,
              cp.MATRIX_COO: oracle.oracle_coo_to_csr}[d.fmt]
        rp, ci, vv, nnz = cp._ip(), cp._ip(), cp._dp(), C.c_int()
        assert fn(C.byref(d), C.byref(rp), C.byref(ci), C.byref(vv), C.byref(nnz)) == 0
        k = nnz.value
        assert np.array_equal(np.ctypeslib.as_array(rp, shape=(d.m + 1,)), want[0])
        if k:
            assert np.array_equal(np.ctypeslib.as_array(ci, shape=(k,)), want[1])
            assert np.array_equal(np.ctypeslib.as_array(vv, shape=(k,)), want[2])


# fields the reference's set_default_parameters leaves unset (src/utils.cu:326-328)
UNSET_BY_REFERENCE = {"grid_size.row_dims", "grid_size.col_dims", "grid_size.decided",
                      "permute_block_size"}


@pytest.mark.parametrize("which", ["library", "oracle"])
def test_default_parameters_match_reference(lib, oracle, golden, which):
    import make_golden
    p = cp.PdhgParameters()
    (lib.set_default_parameters if which == "library" else oracle.oracle_default_parameters)(
        C.byref(p))
    flat = make_golden.flatten(p)
    for name, v in zip(golden["default_names"], golden["default_values"]):
        if str(name) in UNSET_BY_REFERENCE:
            continue
        assert flat[str(name)] == v, name


def test_evaluation_cadence_matches_reference(oracle, golden):
    got = np.array([oracle.oracle_print_frequency(int(t)) for t in golden["pf_iters"]])
    assert np.array_equal(got, golden["pf_values"])


def test_termination_decisions_match_reference(oracle, golden):
    _bind_decisions(oracle)
    eo, ef, ei, il, tl = golden["term_criteria"]
    tc = cp.TerminationCriteria()
    tc.eps_optimal_relative, tc.eps_feasible_relative, tc.eps_infeasible = eo, ef, ei
    tc.iteration_limit, tc.time_sec_limit = int(il), tl
    got = [oracle.oracle_termination_decision(C.byref(tc), *row[:7], int(row[7]), row[8])
           for row in golden["term_inputs"]]
    assert np.array_equal(np.array(got), golden["term_outputs"])
    # every reason of the sweep is exercised
    assert set(np.unique(golden["term_outputs"])) >= {0, 1, 2, 3, 5, 6}


def test_restart_decisions_match_reference(oracle, golden):
    _bind_decisions(oracle)
    art, suff, nec, F = golden["restart_params"]
    rp = cp.RestartParameters()
    rp.artificial_restart_threshold, rp.sufficient_reduction_for_restart = art, suff
    rp.necessary_reduction_for_restart = nec
    got, lasts = [], []
    for row in golden["restart_inputs"]:
        last = C.c_double(row[4])
        got.append(oracle.oracle_restart_decision(C.byref(rp), int(F), int(row[0]), int(row[1]),
                                                  row[2], row[3], C.byref(last)))
        lasts.append(last.value)
    assert np.array_equal(np.array(got), golden["restart_outputs"])
    assert np.array_equal(np.array(lasts), golden["restart_last"])


def test_termination_reason_names_match_reference(lib, golden):
    names = [str(s) for s in golden["reason_names"]]
    assert cp.TERMINATION_REASONS == names
    assert [lib.pdlp_termination_reason_to_string(i).decode() for i in range(8)] == names


# ------------------------------------------------------------ solve checks
def _docs_problem(lib):
    # the reference's documented example (docs/C_API.md:47-90): optimum x=(1,2)
    return cp.Problem.from_csr([0, 2, 3, 5], [0, 1, 1, 0, 1], [1.0, 2.0, 1.0, 3.0, 2.0], 2,
                               c=[1.0, 1.0], lc=[5.0, -np.inf, -np.inf], uc=[5.0, 2.0, 8.0],
                               library=lib)


def test_oracle_solves_documented_example(lib, oracle):
    p = ol.oracle_params(oracle)
    p.termination_criteria.eps_optimal_relative = 1e-8
    p.termination_criteria.eps_feasible_relative = 1e-8
    r, _ = ol.oracle_solve(oracle, _docs_problem(lib), p)
    assert r["status"] == "OPTIMAL"
    np.testing.assert_allclose(r["x"], [1.0, 2.0], atol=1e-6)
    assert abs(r["primal_objective_value"] - 3.0) < 1e-6


def _highs(a):
    from scipy.optimize import linprog
    from scipy.sparse import csr_matrix
    A = csr_matrix((a["vals"], a["col_ind"], a["row_ptr"]), shape=(a["m"], a["n"]))
    lc, uc = a["lc"], a["uc"]
    eq = lc == uc
    ub_rows = ~eq & np.isfinite(uc)
    lb_rows = ~eq & np.isfinite(lc)
    from scipy.sparse import vstack
    A_ub = vstack([A[ub_rows], -A[lb_rows]]).tocsr()
    b_ub = np.concatenate([uc[ub_rows], -lc[lb_rows]])
    res = linprog(a["c"], A_ub=A_ub if A_ub.shape[0] else None,
                  b_ub=b_ub if A_ub.shape[0] else None,
                  A_eq=A[eq] if eq.any() else None, b_eq=lc[eq] if eq.any() else None,
                  bounds=list(zip(np.where(np.isfinite(a["lv"]), a["lv"], None),
                                  np.where(np.isfinite(a["uv"]), a["uv"], None))),
                  method="highs")
    assert res.status == 0, res.message
    return res.fun + a["c0"]


@pytest.mark.parametrize("args", [("random", (60, 150, 600, 11)), ("random", (120, 300, 1500, 12)),
                                  ("transport", (6, 9, 13))])
def test_oracle_matches_highs_at_tight_tolerance(lib, oracle, args):
    pytest.importorskip("scipy")
    prob = cp.Problem.generated(args[0], *args[1], library=lib)
    p = ol.oracle_params(oracle)
    p.termination_criteria.eps_optimal_relative = 1e-8
    p.termination_criteria.eps_feasible_relative = 1e-8
    r, _ = ol.oracle_solve(oracle, prob, p)
    assert r["status"] == "OPTIMAL"
    want = _highs(prob.arrays())
    assert abs(r["primal_objective_value"] - want) <= 1e-6 * (1 + abs(want))
    assert abs(r["dual_objective_value"] - want) <= 1e-6 * (1 + abs(want))


def test_oracle_is_independent_of_thread_count(lib, oracle):
    prob = cp.Problem.generated("random", 200, 500, 2000, 3, library=lib)
    p = ol.oracle_params(oracle)
    r1, t1 = ol.oracle_solve(oracle, prob, p, trace_cap=200, nthreads=1)
    r4, t4 = ol.oracle_solve(oracle, prob, p, trace_cap=200, nthreads=4)
    assert r1["total_count"] == r4["total_count"]
    assert np.array_equal(r1["x"], r4["x"]) and np.array_equal(r1["y"], r4["y"])
    assert np.array_equal(t1, t4)
