"""ctypes access to the test oracle (oracle/liboracle.so) and, where they
were built, to the reference's own host code (oracle/_ref/libref_host.so)
and its own single-GPU solve (oracle/_ref/ref_solve).

Test and benchmark infrastructure only: used by tests/, __graft_entry__.smoke()
and bench.py's baseline arms, never by the product.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess
import tempfile

import numpy as np

import cupdlpx as cp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libref_host.so")
REF_SOLVE = os.path.join(ORACLE_DIR, "_ref", "ref_solve")
# copy of the reference files its single-GPU solve is built from (git-ignored;
# made by `make -C oracle stage` where the reference checkout exists)
REF_STAGE = os.path.join(ROOT, "baseline", "_ref", "D-PDLP")
_dp, _ip = cp._dp, cp._ip
_O = None


def reference_dir() -> str:
    """The reference checkout: $PDLP_REFERENCE_DIR, else the reference_path
    recorded in BASELINE.json at the repository root ("" when neither)."""
    env = os.environ.get("PDLP_REFERENCE_DIR")
    if env:
        return env
    try:
        with open(os.path.join(ROOT, "BASELINE.json")) as f:
            return json.load(f).get("reference_path", "") or ""
    except (OSError, ValueError):
        return ""


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
    O.oracle_generate_random_lp.restype = P
    O.oracle_generate_random_lp.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_ulonglong]
    O.oracle_generate_powerlaw_lp.restype = P
    O.oracle_generate_powerlaw_lp.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_double,
                                              C.c_int, C.c_ulonglong]
    O.oracle_generate_transport_lp.restype = P
    O.oracle_generate_transport_lp.argtypes = [C.c_int, C.c_int, C.c_ulonglong]
    O.oracle_problem_free.restype = None
    O.oracle_problem_free.argtypes = [P]
    _O = O
    return O


class OracleProblem:
    """A seeded LP made by the oracle library's copy of the generators (the
    same problems, bit for bit, as the product's pdlp_generate_*_lp); it has
    the `ptr` / `arrays()` interface of cupdlpx.Problem."""

    def __init__(self, kind: str, *args):
        O = load()
        fn = {"random": O.oracle_generate_random_lp, "powerlaw": O.oracle_generate_powerlaw_lp,
              "transport": O.oracle_generate_transport_lp}[kind]
        self.ptr = fn(*args)
        if not self.ptr:
            raise ValueError(f"generator {kind}{args} failed")
        self._O = O

    def arrays(self) -> dict:
        return cp.problem_arrays(self.ptr)

    def free(self):
        if self.ptr:
            self._O.oracle_problem_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def write_lp_file(problem, path: str) -> None:
    """The problem in ref_solve's input layout (oracle/ref_shim/ref_solve.c)."""
    a = problem.arrays()
    with open(path, "wb") as f:
        f.write(b"PDLPLP1\0")
        np.array([a["m"], a["n"], a["nnz"], 0], dtype="<i4").tofile(f)
        np.array([a["c0"]], dtype="<f8").tofile(f)
        for k in ("c", "lv", "uv", "lc", "uc"):
            np.ascontiguousarray(a[k], dtype="<f8").tofile(f)
        np.ascontiguousarray(a["row_ptr"], dtype="<i4").tofile(f)
        np.ascontiguousarray(a["col_ind"], dtype="<i4").tofile(f)
        np.ascontiguousarray(a["vals"], dtype="<f8").tofile(f)


def build_ref_gpu() -> bool:
    """Build the reference's single-GPU solve from the staged copy (staging it
    first where the reference checkout exists); False when neither exists or
    the build fails."""
    ref = reference_dir()
    if ref and os.path.isdir(os.path.join(ref, "src")):
        r = subprocess.run(["make", "-s", "-C", ORACLE_DIR, "stage", f"REF_DIR={ref}"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            return False
    if not os.path.isdir(os.path.join(REF_STAGE, "src")):
        return False
    r = subprocess.run(["make", "-s", "-j8", "-C", ORACLE_DIR, "refgpu"], capture_output=True,
                       text=True)
    return r.returncode == 0 and os.path.exists(REF_SOLVE)


def ref_gpu_available() -> bool:
    return os.path.exists(REF_SOLVE)


def ref_gpu_solve(problem, eps: float = 1e-4, iter_limit: int = 0, time_limit: float = 0.0,
                  timeout: float | None = None, lp_file: str | None = None) -> dict:
    """One solve by the reference's own single-GPU FP64 code (cuSPARSE/cuBLAS),
    in a fresh process (its power-method start comes from a process-global
    generator).  Returns the result scalars, `wall_s` (the solve_lp_problem
    call) and the x, y, rc vectors.  `lp_file` reuses an LP file already
    written by write_lp_file."""
    if not ref_gpu_available():
        raise RuntimeError("the reference's single-GPU solve is not built")
    with tempfile.TemporaryDirectory() as d:
        lp = lp_file
        if lp is None:
            lp = os.path.join(d, "lp.bin")
            write_lp_file(problem, lp)
        out = os.path.join(d, "out.bin")
        cmd = [REF_SOLVE, lp, out, "--eps", repr(eps)]
        if iter_limit > 0:
            cmd += ["--iter-limit", str(iter_limit)]
        if time_limit > 0:
            cmd += ["--time-limit", repr(time_limit)]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"ref_solve failed ({r.returncode}): {r.stderr[-2000:]}")
        line = [ln for ln in r.stdout.splitlines() if ln.startswith("REF_RESULT ")][-1]
        res = json.loads(line[len("REF_RESULT "):])
        v = np.fromfile(out, dtype="<f8")
        n, m = res["n"], res["m"]
        res["x"], res["y"], res["rc"] = v[:n].copy(), v[n:n + m].copy(), v[n + m:].copy()
        return res


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
