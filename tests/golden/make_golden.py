"""Write tests/golden/ref_host.npz: outputs of the reference's own host code.

The reference's host-side C/C++ (rescaling, input converters, defaults,
evaluation cadence, termination and restart tests, reason names) is compiled
in place by ``make -C oracle ref`` into oracle/_ref/libref_host.so.  This
script runs it on small stored inputs and saves inputs and outputs, so that
the oracle can be checked against the reference on any machine, including
ones without the reference sources.

Run (where the reference sources exist):
    make -C oracle ref && python tests/golden/make_golden.py
    python tests/golden/make_golden.py mps     # ref_mps.npz: read_mps_file on tests/golden/mps
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "d-pdlp_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import cupdlpx as cp  # noqa: E402
import oracle_lib as ol  # noqa: E402

OUT = os.path.join(HERE, "ref_host.npz")

# small seeded LPs from the library's generators: (kind, args)
LPS = [("random", (50, 80, 300, 3)), ("random", (300, 100, 2000, 5)),
       ("random", (400, 1000, 4000, 7)), ("transport", (3, 4, 2))]
# (l_inf_ruiz_iterations, has_pock_chambolle_alpha, pock_chambolle_alpha,
#  bound_objective_rescaling)
RESCALE_SETS = [(10, True, 1.0, True), (0, True, 1.0, True), (3, False, 1.0, False),
                (5, True, 0.5, True)]
RESCALE_KEYS = ("vals", "c", "lv", "uv", "lc", "uc", "con", "var")


def flatten(st, prefix="") -> dict:
    """Every scalar field of a ctypes structure, nested names joined by '.'."""
    out = {}
    for name, typ in st._fields_:
        v = getattr(st, name)
        if isinstance(v, C.Structure):
            out.update(flatten(v, prefix + name + "."))
        else:
            out[prefix + name] = float(v)
    return out


def converter_cases():
    """Dense, CSC and COO inputs exercising the zero tolerance and ordering."""
    dense = np.array([[1.0, 0.0, 2e-13, -3.0, 0.0],
                      [0.0, 0.0, 0.0, 0.0, 0.0],
                      [5e-12, 4.0, 0.0, 0.0, -1e-14],
                      [0.0, -2.5, 7.0, 0.0, 1.0]])
    cases = []
    for tol in (0.0, 1e-12):
        cases.append(("dense", tol, {"A": dense}))
    # CSC of a 3x4 matrix (column pointers, row indices, values)
    csc = {"col_ptr": np.array([0, 2, 2, 4, 5], np.int32),
           "row_ind": np.array([0, 2, 1, 2, 0], np.int32),
           "vals": np.array([1.5, -2.0, 3.0, 1e-13, 4.0])}
    for tol in (0.0, 1e-12):
        cases.append(("csc", tol, csc))
    coo = {"row_ind": np.array([2, 0, 1, 0, 2, 1], np.int32),
           "col_ind": np.array([1, 3, 0, 0, 3, 2], np.int32),
           "vals": np.array([4.0, -1.0, 2.0, 3.0, 1e-13, -6.0])}
    for tol in (0.0, 1e-12):
        cases.append(("coo", tol, coo))
    return cases


def desc_for(kind, tol, data):
    """A matrix_desc_t over `data`; the returned list keeps the arrays it
    points to alive."""
    d = cp.MatrixDesc()
    d.zero_tolerance = tol
    keep = [data]
    if kind == "dense":
        A = np.ascontiguousarray(data["A"])
        d.m, d.n, d.fmt = A.shape[0], A.shape[1], cp.MATRIX_DENSE
        d.data.dense.A = cp.as_dp(A)
        keep.append(A)
    elif kind == "csc":
        d.m, d.n, d.fmt = 3, 4, cp.MATRIX_CSC
        d.data.csc.nnz = len(data["vals"])
        d.data.csc.col_ptr = cp.as_ip(data["col_ptr"])
        d.data.csc.row_ind = cp.as_ip(data["row_ind"])
        d.data.csc.vals = cp.as_dp(data["vals"])
    else:
        d.m, d.n, d.fmt = 3, 4, cp.MATRIX_COO
        d.data.coo.nnz = len(data["vals"])
        d.data.coo.row_ind = cp.as_ip(data["row_ind"])
        d.data.coo.col_ind = cp.as_ip(data["col_ind"])
        d.data.coo.vals = cp.as_dp(data["vals"])
    return d, keep


def termination_sweep(rng, n=3000):
    eps = 1e-4
    pick = lambda opts: np.array([opts[i] for i in rng.integers(0, len(opts), n)])
    near = [0.0, 0.5 * eps, eps, 2 * eps, 1.0]
    X = np.stack([
        pick(near), pick(near), pick(near),                             # rel_p rel_d rel_gap
        pick([-1.0, 0.0, 1e-3, 1.0]), pick([0.0, 1e-12, 1e-10, 1e-6]),  # dray_obj max_dray
        pick([-1.0, 0.0, -1e-3, 1.0]), pick([0.0, 1e-12, 1e-10, 1e-6]),  # pray_obj max_pray
        pick([0, 999, 1000, 1001]), pick([0.0, 9.9, 10.0, 11.0]),        # total cum_time
    ], axis=1)
    return X


def restart_sweep(rng, n=3000):
    pick = lambda opts: np.array([opts[i] for i in rng.integers(0, len(opts), n)])
    return np.stack([
        pick([100, 199, 200, 201, 400, 1000]),                # total
        pick([0, 50, 72, 73, 144, 360, 400]),                 # inner
        pick([0.0, 0.1, 0.2, 0.3, 0.5, 0.6, 1.0]),            # fpe
        pick([1.0, 0.5, 2.0]),                                # initial fpe
        pick([np.inf, 0.05, 0.25, 0.5, 1.0]),                 # last trial fpe
    ], axis=1)


def main():
    O = ol.load()
    R = ol.load_ref()
    if R is None:
        sys.exit("oracle/_ref/libref_host.so is missing: run make -C oracle ref")
    L = cp.lib()
    R.ref_h_termination.restype = C.c_int
    R.ref_h_termination.argtypes = [C.POINTER(cp.TerminationCriteria)] + [C.c_double] * 7 + [
        C.c_int, C.c_double]
    R.ref_h_restart.restype = C.c_int
    R.ref_h_restart.argtypes = [C.POINTER(cp.RestartParameters), C.c_int, C.c_int, C.c_int,
                                C.c_double, C.c_double, cp._dp]
    R.termination_reason_to_string.restype = C.c_char_p
    R.termination_reason_to_string.argtypes = [C.c_int]
    g = {}
    # rescaling
    for i, (kind, args) in enumerate(LPS):
        prob = cp.Problem.generated(kind, *args, library=L)
        a = prob.arrays()
        for k in ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv"):
            g[f"lp{i}_{k}"] = a[k]
        g[f"lp{i}_n"] = np.array(a["n"])
        for j, (ruiz, pc, alpha, bo) in enumerate(RESCALE_SETS):
            p = ol.oracle_params(O)
            p.l_inf_ruiz_iterations, p.has_pock_chambolle_alpha = ruiz, pc
            p.pock_chambolle_alpha, p.bound_objective_rescaling = alpha, bo
            r = ol.ref_rescale(R, prob, p)
            for k in RESCALE_KEYS:
                g[f"resc{i}_{j}_{k}"] = r[k]
            g[f"resc{i}_{j}_cbob"] = np.array([r["cb"], r["ob"]])
    g["rescale_sets"] = np.array(RESCALE_SETS, dtype=np.float64)
    # converters: the reference's create_lp_problem on dense / CSC / COO input
    for i, (kind, tol, data) in enumerate(converter_cases()):
        d, keep = desc_for(kind, tol, data)
        n, m = d.n, d.m
        c = np.zeros(n)
        pp = R.create_lp_problem(cp.as_dp(c), C.byref(d), None, None, None, None, None)
        a = cp.problem_arrays(pp)
        g[f"conv{i}_row_ptr"], g[f"conv{i}_col_ind"], g[f"conv{i}_vals"] = (
            a["row_ptr"], a["col_ind"], a["vals"])
        g[f"conv{i}_lc"], g[f"conv{i}_uc"] = a["lc"], a["uc"]
        g[f"conv{i}_lv"], g[f"conv{i}_uv"] = a["lv"], a["uv"]
        R.lp_problem_free(pp)
    # defaults
    p = cp.PdhgParameters()
    R.set_default_parameters(C.byref(p))
    flat = flatten(p)
    g["default_names"] = np.array(sorted(flat))
    g["default_values"] = np.array([flat[k] for k in sorted(flat)])
    # evaluation cadence
    iters = np.unique(np.concatenate([np.arange(0, 2100), np.arange(0, 200001, 97),
                                      [9999, 10000, 10001, 99999, 100000, 100001]]))
    g["pf_iters"] = iters.astype(np.int64)
    g["pf_values"] = np.array([R.get_print_frequency(int(t)) for t in iters], np.int64)
    # termination and restart decisions
    rng = np.random.default_rng(2024)
    tc = cp.TerminationCriteria()
    tc.eps_optimal_relative = tc.eps_feasible_relative = 1e-4
    tc.eps_infeasible = 1e-10
    tc.iteration_limit = 1000
    tc.time_sec_limit = 10.0
    X = termination_sweep(rng)
    g["term_inputs"] = X
    g["term_criteria"] = np.array([1e-4, 1e-4, 1e-10, 1000, 10.0])
    g["term_outputs"] = np.array([R.ref_h_termination(C.byref(tc), *row[:7], int(row[7]), row[8])
                                  for row in X], np.int64)
    rp = cp.RestartParameters()
    rp.artificial_restart_threshold, rp.sufficient_reduction_for_restart = 0.36, 0.2
    rp.necessary_reduction_for_restart = 0.5
    Y = restart_sweep(rng)
    outs, lasts = [], []
    for row in Y:
        last = C.c_double(row[4])
        outs.append(R.ref_h_restart(C.byref(rp), 200, int(row[0]), int(row[1]), row[2], row[3],
                                    C.byref(last)))
        lasts.append(last.value)
    g["restart_inputs"], g["restart_outputs"] = Y, np.array(outs, np.int64)
    g["restart_last"] = np.array(lasts)
    g["restart_params"] = np.array([0.36, 0.2, 0.5, 200])
    g["reason_names"] = np.array([R.termination_reason_to_string(i).decode() for i in range(8)])
    np.savez_compressed(OUT, **g)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes, {len(g)} arrays)")


if __name__ == "__main__" and len(sys.argv) == 1:
    main()


# ------------------------------------------------------------------ MPS
MPS_DIR = os.path.join(HERE, "mps")
MPS_OUT = os.path.join(HERE, "ref_mps.npz")


def mps_main():
    """The reference's read_mps_file on every fixture under tests/golden/mps."""
    R = ol.load_ref()
    if R is None:
        sys.exit("oracle/_ref/libref_host.so is missing: run make -C oracle ref")
    R.read_mps_file.restype = C.POINTER(cp.LpProblem)
    R.read_mps_file.argtypes = [C.c_char_p]
    g = {}
    names = sorted(f for f in os.listdir(MPS_DIR) if ".mps" in f)
    for name in names:
        pp = R.read_mps_file(os.path.join(MPS_DIR, name).encode())
        if not pp:
            g[f"{name}__failed"] = np.array(1)
            continue
        a = cp.problem_arrays(pp)
        for k in ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv"):
            g[f"{name}__{k}"] = a[k]
        g[f"{name}__shape"] = np.array([a["m"], a["n"], a["nnz"]])
        g[f"{name}__c0"] = np.array(a["c0"])
        R.lp_problem_free(pp)
    g["names"] = np.array(names)
    np.savez_compressed(MPS_OUT, **g)
    print(f"wrote {MPS_OUT} ({len(names)} files)")


if __name__ == "__main__" and len(sys.argv) > 1 and sys.argv[1] == "mps":
    mps_main()
