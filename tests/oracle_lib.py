"""ctypes access to the test oracle (oracle/liboracle.so) and, where it was
built, to the reference's own host code (oracle/_ref/libref_host.so).

Test infrastructure only: used by tests/, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

import cupdlpx as cp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libref_host.so")
_dp, _ip = cp._dp, cp._ip
_O = None


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)


def load():
    global _O
    if _O is not None:
        return _O
    if not os.path.exists(ORACLE_SO):
        build_oracle()
    O = C.CDLL(ORACLE_SO)
    P, R, PP = C.POINTER(cp.LpProblem), C.POINTER(cp.Result), C.POINTER(cp.PdhgParameters)
    O.oracle_solve.restype = R
    O.oracle_solve.argtypes = [P, PP, C.c_int, _dp, C.c_int, _ip]
    O.oracle_result_free.argtypes = [R]
    O.oracle_default_parameters.argtypes = [PP]
    O.oracle_rescale.argtypes = [P, PP] + [_dp] * 8 + [_dp, _dp]
    O.oracle_transpose.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
    O.oracle_spmv.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_int]
    O.oracle_power_method.restype = C.c_double
    O.oracle_power_method.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, C.c_int, C.c_double,
                                      _ip, C.c_int]
    O.oracle_power_start_vector.argtypes = [C.c_int, _dp]
    for f in ("oracle_dense_to_csr", "oracle_csc_to_csr", "oracle_coo_to_csr"):
        getattr(O, f).restype = C.c_int
        getattr(O, f).argtypes = [C.POINTER(cp.MatrixDesc), C.POINTER(_ip), C.POINTER(_ip),
                                  C.POINTER(_dp), _ip]
    O.oracle_print_frequency.restype = C.c_int
    O.oracle_print_frequency.argtypes = [C.c_int]
    _O = O
    return O


class RescaleInfo(C.Structure):
    """Reference rescale_info_t (internal/internal_types.h:147-154)."""
    _fields_ = [("scaled_problem", C.POINTER(cp.LpProblem)), ("con_rescale", _dp),
                ("var_rescale", _dp), ("con_bound_rescale", C.c_double),
                ("obj_vec_rescale", C.c_double), ("rescaling_time_sec", C.c_double)]


def load_ref():
    """The reference's host code, or None when it was not built here."""
    if not os.path.exists(REF_SO):
        return None
    R = C.CDLL(REF_SO)
    cp.declare_api(R)
    R.rescale_problem.restype = C.POINTER(RescaleInfo)
    R.rescale_problem.argtypes = [C.POINTER(cp.PdhgParameters), C.POINTER(cp.LpProblem)]
    R.get_print_frequency.restype = C.c_int
    R.get_print_frequency.argtypes = [C.c_int]
    return R


def oracle_params(O) -> cp.PdhgParameters:
    p = cp.PdhgParameters()
    O.oracle_default_parameters(C.byref(p))
    p.presolve = False
    return p


def oracle_solve(O, problem: "cp.Problem", params=None, trace_cap: int = 0, nthreads: int = 0):
    tr = np.zeros((max(trace_cap, 1), cp.TRACE_WIDTH))
    tl = C.c_int(0)
    p = params if params is not None else oracle_params(O)
    r = O.oracle_solve(problem.ptr, C.byref(p), nthreads, cp.as_dp(tr) if trace_cap else None,
                       trace_cap, C.byref(tl))
    try:
        res = cp.result_dict(r)
    finally:
        O.oracle_result_free(r)
    return res, tr[: tl.value].copy()


def oracle_rescale(O, problem: "cp.Problem", params) -> dict:
    a = problem.arrays()
    m, n, nnz = a["m"], a["n"], a["nnz"]
    out = {k: np.zeros(s) for k, s in (("vals", nnz), ("c", n), ("lv", n), ("uv", n), ("lc", m),
                                       ("uc", m), ("con", m), ("var", n))}
    cb, ob = C.c_double(), C.c_double()
    O.oracle_rescale(problem.ptr, C.byref(params), *[cp.as_dp(out[k]) for k in
                     ("vals", "c", "lv", "uv", "lc", "uc", "con", "var")], C.byref(cb), C.byref(ob))
    out["cb"], out["ob"] = cb.value, ob.value
    return out


def ref_rescale(R, problem: "cp.Problem", params) -> dict:
    info = R.rescale_problem(C.byref(params), problem.ptr).contents
    sp = cp.problem_arrays(info.scaled_problem)
    m, n = sp["m"], sp["n"]
    return {"vals": sp["vals"], "c": sp["c"], "lv": sp["lv"], "uv": sp["uv"], "lc": sp["lc"],
            "uc": sp["uc"],
            "con": np.ctypeslib.as_array(info.con_rescale, shape=(m,)).copy() if m else np.zeros(0),
            "var": np.ctypeslib.as_array(info.var_rescale, shape=(n,)).copy() if n else np.zeros(0),
            "cb": info.con_bound_rescale, "ob": info.obj_vec_rescale}
