"""ctypes binding of the GB300 PDHG solver's C API.

This is the binding a Python caller of the reference's C API
(``include/cupdlpx.h``) would write; the structures mirror
``include/cupdlpx_types.h`` field for field.  No PyTorch is involved: the
library takes host arrays and returns host arrays.

The CUDA library must be built (``build.py``); loading fails loudly when it
is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcupdlpx_gb300.so")

# --------------------------------------------------------------- structures
TERMINATION_REASONS = [
    "UNSPECIFIED", "OPTIMAL", "PRIMAL_INFEASIBLE", "DUAL_INFEASIBLE",
    "INFEASIBLE_OR_UNBOUNDED", "TIME_LIMIT", "ITERATION_LIMIT", "FEAS_POLISH_SUCCESS",
]
NORM_L2, NORM_LINF = 0, 1
MATRIX_DENSE, MATRIX_CSR, MATRIX_CSC, MATRIX_COO = 0, 1, 2, 3
TRACE_WIDTH = 10
TRACE_FIELDS = ["iter", "rel_primal", "rel_dual", "rel_gap", "primal_obj", "dual_obj",
                "primal_weight", "fixed_point_error", "step_size", "inner_count"]

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class LpProblem(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("variable_lower_bound", _dp),
        ("variable_upper_bound", _dp),
        ("objective_vector", _dp),
        ("objective_constant", C.c_double),
        ("constraint_matrix_row_pointers", _ip),
        ("constraint_matrix_col_indices", _ip),
        ("constraint_matrix_values", _dp),
        ("constraint_matrix_num_nonzeros", C.c_int),
        ("constraint_lower_bound", _dp),
        ("constraint_upper_bound", _dp),
        ("primal_start", _dp),
        ("dual_start", _dp),
    ]


class RestartParameters(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "artificial_restart_threshold", "sufficient_reduction_for_restart",
        "necessary_reduction_for_restart", "k_p", "k_i", "k_d", "i_smooth")]


class TerminationCriteria(C.Structure):
    _fields_ = [
        ("eps_optimal_relative", C.c_double),
        ("eps_feasible_relative", C.c_double),
        ("eps_feas_polish_relative", C.c_double),
        ("eps_infeasible", C.c_double),
        ("time_sec_limit", C.c_double),
        ("iteration_limit", C.c_int),
    ]


class GridSize(C.Structure):
    _fields_ = [("row_dims", C.c_int), ("col_dims", C.c_int), ("decided", C.c_bool)]


class PdhgParameters(C.Structure):
    _fields_ = [
        ("l_inf_ruiz_iterations", C.c_int),
        ("has_pock_chambolle_alpha", C.c_bool),
        ("pock_chambolle_alpha", C.c_double),
        ("bound_objective_rescaling", C.c_bool),
        ("verbose", C.c_bool),
        ("termination_evaluation_frequency", C.c_int),
        ("sv_max_iter", C.c_int),
        ("sv_tol", C.c_double),
        ("termination_criteria", TerminationCriteria),
        ("restart_params", RestartParameters),
        ("reflection_coefficient", C.c_double),
        ("feasibility_polishing", C.c_bool),
        ("optimality_norm", C.c_int),
        ("presolve", C.c_bool),
        ("partition_method", C.c_int),
        ("permute_method", C.c_int),
        ("grid_size", GridSize),
        ("permute_block_size", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("num_variables", C.c_int),
        ("num_constraints", C.c_int),
        ("num_nonzeros", C.c_int),
        ("num_reduced_variables", C.c_int),
        ("num_reduced_constraints", C.c_int),
        ("num_reduced_nonzeros", C.c_int),
        ("primal_solution", _dp),
        ("dual_solution", _dp),
        ("reduced_cost", _dp),
        ("total_count", C.c_int),
        ("rescaling_time_sec", C.c_double),
        ("cumulative_time_sec", C.c_double),
        ("presolve_time", C.c_double),
        ("presolve_status", C.c_int),
        ("absolute_primal_residual", C.c_double),
        ("relative_primal_residual", C.c_double),
        ("absolute_dual_residual", C.c_double),
        ("relative_dual_residual", C.c_double),
        ("primal_objective_value", C.c_double),
        ("dual_objective_value", C.c_double),
        ("objective_gap", C.c_double),
        ("relative_objective_gap", C.c_double),
        ("max_primal_ray_infeasibility", C.c_double),
        ("max_dual_ray_infeasibility", C.c_double),
        ("primal_ray_linear_objective", C.c_double),
        ("dual_ray_objective", C.c_double),
        ("termination_reason", C.c_int),
        ("feasibility_polishing_time", C.c_double),
        ("feasibility_iteration", C.c_int),
    ]


class _Dense(C.Structure):
    _fields_ = [("A", _dp)]


class _Csr(C.Structure):
    _fields_ = [("nnz", C.c_int), ("row_ptr", _ip), ("col_ind", _ip), ("vals", _dp)]


class _Csc(C.Structure):
    _fields_ = [("nnz", C.c_int), ("col_ptr", _ip), ("row_ind", _ip), ("vals", _dp)]


class _Coo(C.Structure):
    _fields_ = [("nnz", C.c_int), ("row_ind", _ip), ("col_ind", _ip), ("vals", _dp)]


class _MatrixData(C.Union):
    _fields_ = [("dense", _Dense), ("csr", _Csr), ("csc", _Csc), ("coo", _Coo)]


class MatrixDesc(C.Structure):
    _fields_ = [
        ("m", C.c_int),
        ("n", C.c_int),
        ("fmt", C.c_int),
        ("zero_tolerance", C.c_double),
        ("data", _MatrixData),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("power_iterations", C.c_int),
        ("sigma_max", C.c_double),
        ("setup_seconds", C.c_double),
        ("rescale_seconds", C.c_double),
        ("power_seconds", C.c_double),
        ("loop_seconds", C.c_double),
        ("total_seconds", C.c_double),
        ("graphs", C.c_int),
        ("kernel_launches", C.c_longlong),
        ("device_seconds", C.c_double),
        ("refinement_rounds", C.c_int),
        ("precision", C.c_int),
        ("primal_step_ms", C.c_double),
        ("dual_step_ms", C.c_double),
        ("timed_chunks", C.c_int),
        ("fp64_finish", C.c_int),
        ("spmv_kernel_A", C.c_int),
        ("spmv_kernel_AT", C.c_int),
        ("tune_ms", C.c_double * 4),
    ]


PRECISION_FP64, PRECISION_FP32_REFINE, PRECISION_FP32_MATRIX = 0, 1, 2


def info_dict(info) -> dict:
    """pdlp_solve_info_t as a dict (arrays as lists)."""
    out = {}
    for f, _ in SolveInfo._fields_:
        v = getattr(info, f)
        out[f] = list(v) if hasattr(v, "__len__") else v
    return out


class RequestInfo(C.Structure):
    _fields_ = [("queued_seconds", C.c_double), ("solve_seconds", C.c_double),
                ("latency_seconds", C.c_double), ("worker", C.c_int),
                ("device_bytes", C.c_longlong), ("upload_seconds", C.c_double),
                ("device_seconds", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_longlong), ("failed", C.c_longlong),
                ("queued", C.c_longlong), ("in_flight", C.c_int), ("max_in_flight", C.c_int),
                ("iterations", C.c_longlong), ("device_bytes_in_use", C.c_longlong),
                ("busy_seconds", C.c_double), ("rejected", C.c_longlong),
                ("queued_host_bytes", C.c_longlong)]


class BatchInfo(C.Structure):
    _fields_ = [("lps", C.c_int), ("failed", C.c_int), ("wall_seconds", C.c_double),
                ("lps_per_second", C.c_double), ("iterations", C.c_longlong),
                ("max_concurrent", C.c_int)]


class Options(C.Structure):
    _fields_ = [("precision", C.c_int), ("max_refinements", C.c_int), ("inner_eps", C.c_double)]


# -------------------------------------------------------------- prototypes
def declare_api(lib: C.CDLL) -> C.CDLL:
    """Attach argtypes/restype of the six reference entry points."""
    P, R = C.POINTER(LpProblem), C.POINTER(Result)
    lib.create_lp_problem.restype = P
    lib.create_lp_problem.argtypes = [_dp, C.POINTER(MatrixDesc), _dp, _dp, _dp, _dp, _dp]
    lib.set_start_values.restype = None
    lib.set_start_values.argtypes = [P, _dp, _dp]
    lib.solve_lp_problem.restype = R
    lib.solve_lp_problem.argtypes = [P, C.POINTER(PdhgParameters)]
    lib.set_default_parameters.restype = None
    lib.set_default_parameters.argtypes = [C.POINTER(PdhgParameters)]
    lib.cupdlpx_result_free.restype = None
    lib.cupdlpx_result_free.argtypes = [R]
    lib.lp_problem_free.restype = None
    lib.lp_problem_free.argtypes = [P]
    return lib


def _declare_ext(lib: C.CDLL) -> None:
    P, R = C.POINTER(LpProblem), C.POINTER(Result)
    lib.pdlp_solve_ex.restype = R
    lib.pdlp_solve_ex.argtypes = [P, C.POINTER(PdhgParameters), _dp, C.c_int, _ip,
                                  C.POINTER(SolveInfo)]
    lib.pdlp_last_error.restype = C.c_char_p
    lib.pdlp_termination_reason_to_string.restype = C.c_char_p
    lib.pdlp_termination_reason_to_string.argtypes = [C.c_int]
    lib.pdlp_generate_random_lp.restype = P
    lib.pdlp_generate_random_lp.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_ulonglong]
    lib.pdlp_generate_powerlaw_lp.restype = P
    lib.pdlp_generate_powerlaw_lp.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_double,
                                              C.c_int, C.c_ulonglong]
    lib.pdlp_generate_transport_lp.restype = P
    lib.pdlp_generate_transport_lp.argtypes = [C.c_int, C.c_int, C.c_ulonglong]
    lib.pdlp_gpu_rescale.restype = C.c_int
    lib.pdlp_gpu_rescale.argtypes = [P, C.POINTER(PdhgParameters)] + [_dp] * 8 + [_dp, _dp]
    lib.pdlp_gpu_spmv.restype = C.c_int
    lib.pdlp_gpu_spmv.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_int]
    lib.pdlp_gpu_spmv_variant.restype = C.c_int
    lib.pdlp_gpu_spmv_variant.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _dp, _dp, C.c_int,
                                          C.c_int]
    lib.pdlp_spmv_plan.restype = C.c_int
    lib.pdlp_spmv_plan.argtypes = [C.c_int, _ip, C.c_int, C.c_int, _ip, C.c_int, _ip, _ip, _ip]
    lib.pdlp_gpu_transpose.restype = C.c_int
    lib.pdlp_gpu_transpose.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
    lib.pdlp_spmv_pipe_plan.restype = C.c_int
    lib.pdlp_spmv_pipe_plan.argtypes = [C.c_int, _ip, C.c_int, _ip, _ip, C.c_int, _ip, _ip, _ip]
    lib.pdlp_host_transpose.restype = C.c_int
    lib.pdlp_host_transpose.argtypes = [C.c_int, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
    lib.pdlp_gpu_power_method.restype = C.c_int
    lib.pdlp_gpu_power_method.argtypes = [P, C.POINTER(PdhgParameters), _dp, _ip]
    lib.pdlp_device_problem_create.restype = C.c_void_p
    lib.pdlp_device_problem_create.argtypes = [P]
    lib.pdlp_device_problem_free.restype = None
    lib.pdlp_device_problem_free.argtypes = [C.c_void_p]
    lib.pdlp_device_problem_bytes.restype = C.c_longlong
    lib.pdlp_device_problem_bytes.argtypes = [C.c_void_p]
    lib.pdlp_device_problem_solve.restype = R
    lib.pdlp_device_problem_solve.argtypes = [C.c_void_p, C.POINTER(PdhgParameters),
                                              C.POINTER(SolveInfo)]
    lib.pdlp_solve_opts.restype = R
    lib.pdlp_solve_opts.argtypes = [P, C.POINTER(PdhgParameters), C.POINTER(Options),
                                    C.POINTER(SolveInfo)]
    lib.pdlp_device_problem_solve_opts.restype = R
    lib.pdlp_device_problem_solve_opts.argtypes = [C.c_void_p, C.POINTER(PdhgParameters),
                                                   C.POINTER(Options), C.POINTER(SolveInfo)]
    lib.pdlp_device_problem_time_kernels_prec.restype = C.c_int
    lib.pdlp_device_problem_time_kernels_prec.argtypes = [C.c_void_p, C.POINTER(PdhgParameters),
                                                          C.c_int, C.c_int, _dp]
    lib.pdlp_problem_wire_size.restype = C.c_longlong
    lib.pdlp_problem_wire_size.argtypes = [P]
    lib.pdlp_problem_serialize.restype = C.c_longlong
    lib.pdlp_problem_serialize.argtypes = [P, C.c_void_p, C.c_longlong]
    lib.pdlp_problem_deserialize.restype = P
    lib.pdlp_problem_deserialize.argtypes = [C.c_void_p, C.c_longlong]
    lib.pdlp_server_submit_bytes.restype = C.c_longlong
    lib.pdlp_server_submit_bytes.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong]
    lib.read_mps_file.restype = P
    lib.read_mps_file.argtypes = [C.c_char_p]
    lib.pdlp_estimate_device_bytes.restype = C.c_longlong
    lib.pdlp_estimate_device_bytes.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_int]
    lib.pdlp_server_create.restype = C.c_void_p
    lib.pdlp_server_create.argtypes = [C.POINTER(PdhgParameters), C.POINTER(Options), C.c_int,
                                       C.c_longlong]
    lib.pdlp_server_submit.restype = C.c_longlong
    lib.pdlp_server_submit.argtypes = [C.c_void_p, P]
    lib.pdlp_server_wait.restype = R
    lib.pdlp_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(RequestInfo)]
    lib.pdlp_server_stats.restype = C.c_int
    lib.pdlp_server_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    lib.pdlp_server_set_queue_limit.restype = C.c_int
    lib.pdlp_server_set_queue_limit.argtypes = [C.c_void_p, C.c_longlong]
    lib.pdlp_server_destroy.restype = None
    lib.pdlp_server_destroy.argtypes = [C.c_void_p]
    lib.pdlp_batch_solve.restype = C.c_int
    lib.pdlp_batch_solve.argtypes = [C.POINTER(P), C.c_int, C.POINTER(PdhgParameters),
                                     C.POINTER(Options), C.c_int, C.c_longlong, C.POINTER(R),
                                     C.POINTER(BatchInfo)]
    lib.pdlp_release_pooled_memory.restype = None
    lib.pdlp_release_pooled_memory.argtypes = []
    lib.pdlp_device_problem_time_kernels.restype = C.c_int
    lib.pdlp_device_problem_time_kernels.argtypes = [C.c_void_p, C.POINTER(PdhgParameters),
                                                     C.c_int, _dp]


_LIB: C.CDLL | None = None


def lib() -> C.CDLL:
    """The loaded solver library (raises if it has not been built)."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run d-pdlp_gb300/build.py "
                               "(the CUDA solver has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        declare_api(L)
        _declare_ext(L)
        _LIB = L
    return _LIB


# ------------------------------------------------------------------ helpers
def as_dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def as_ip(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


def default_parameters(library: C.CDLL | None = None) -> PdhgParameters:
    p = PdhgParameters()
    (library or lib()).set_default_parameters(C.byref(p))
    return p


def problem_arrays(p) -> dict:
    """Copy an lp_problem_t (pointer or struct) into numpy arrays."""
    s = p.contents if hasattr(p, "contents") else p
    m, n, nnz = s.num_constraints, s.num_variables, s.constraint_matrix_num_nonzeros

    def cp(ptr, k, dt):
        if k == 0:
            return np.zeros(0, dtype=dt)
        return np.ctypeslib.as_array(ptr, shape=(k,)).copy().astype(dt, copy=False)

    return {
        "m": m, "n": n, "nnz": nnz,
        "row_ptr": cp(s.constraint_matrix_row_pointers, m + 1, np.int32),
        "col_ind": cp(s.constraint_matrix_col_indices, nnz, np.int32),
        "vals": cp(s.constraint_matrix_values, nnz, np.float64),
        "c": cp(s.objective_vector, n, np.float64),
        "lv": cp(s.variable_lower_bound, n, np.float64),
        "uv": cp(s.variable_upper_bound, n, np.float64),
        "lc": cp(s.constraint_lower_bound, m, np.float64),
        "uc": cp(s.constraint_upper_bound, m, np.float64),
        "c0": s.objective_constant,
    }


def result_dict(r) -> dict:
    s = r.contents
    n, m = s.num_variables, s.num_constraints
    out = {f: getattr(s, f) for f, _ in Result._fields_
           if f not in ("primal_solution", "dual_solution", "reduced_cost")}
    out["x"] = np.ctypeslib.as_array(s.primal_solution, shape=(n,)).copy() if n else np.zeros(0)
    out["y"] = np.ctypeslib.as_array(s.dual_solution, shape=(m,)).copy() if m else np.zeros(0)
    out["rc"] = np.ctypeslib.as_array(s.reduced_cost, shape=(n,)).copy() if n else np.zeros(0)
    out["status"] = TERMINATION_REASONS[s.termination_reason]
    return out


class Problem:
    """Owns an lp_problem_t made by create_lp_problem (or a generator)."""

    def __init__(self, ptr, library: C.CDLL | None = None):
        if not ptr:
            raise ValueError("problem construction failed: "
                             + (library or lib()).pdlp_last_error().decode())
        self.ptr = ptr
        self._lib = library or lib()

    @classmethod
    def from_csr(cls, row_ptr, col_ind, vals, n, c=None, lc=None, uc=None, lv=None,
                 uv=None, c0=None, library: C.CDLL | None = None) -> "Problem":
        L = library or lib()
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int32)
        col_ind = np.ascontiguousarray(col_ind, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        d = MatrixDesc()
        d.m, d.n, d.fmt, d.zero_tolerance = len(row_ptr) - 1, n, MATRIX_CSR, 0.0
        d.data.csr.nnz = len(vals)
        d.data.csr.row_ptr, d.data.csr.col_ind, d.data.csr.vals = (
            as_ip(row_ptr), as_ip(col_ind), as_dp(vals))
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        arrs = [conv(a) for a in (c, lc, uc, lv, uv)]
        k0 = None if c0 is None else C.byref(C.c_double(c0))
        ptr = L.create_lp_problem(as_dp(arrs[0]), C.byref(d), as_dp(arrs[1]), as_dp(arrs[2]),
                                  as_dp(arrs[3]), as_dp(arrs[4]), k0)
        return cls(ptr, L)

    @classmethod
    def from_mps(cls, path: str, library: C.CDLL | None = None) -> "Problem":
        """read_mps_file (free-format MPS, .mps or .mps.gz)."""
        L = library or lib()
        ptr = L.read_mps_file(os.fsencode(path))
        if not ptr:
            raise ValueError(f"cannot read MPS file {path}")
        return cls(ptr, L)

    @classmethod
    def generated(cls, kind: str, *args, library: C.CDLL | None = None) -> "Problem":
        L = library or lib()
        fn = {"random": L.pdlp_generate_random_lp, "powerlaw": L.pdlp_generate_powerlaw_lp,
              "transport": L.pdlp_generate_transport_lp}[kind]
        return cls(fn(*args), L)

    def arrays(self) -> dict:
        return problem_arrays(self.ptr)

    def to_bytes(self) -> bytes:
        """The problem in the binary request format (pdlp_problem_serialize)."""
        size = self._lib.pdlp_problem_wire_size(self.ptr)
        buf = C.create_string_buffer(max(int(size), 1))
        if self._lib.pdlp_problem_serialize(self.ptr, buf, size) != size:
            raise RuntimeError("serialize failed")
        return buf.raw[:size]

    @classmethod
    def from_bytes(cls, data: bytes, library: C.CDLL | None = None) -> "Problem":
        L = library or lib()
        ptr = L.pdlp_problem_deserialize(data, len(data))
        if not ptr:
            raise ValueError("malformed problem payload")
        return cls(ptr, L)

    def set_start(self, x=None, y=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        xs, ys = conv(x), conv(y)
        self._lib.set_start_values(self.ptr, as_dp(xs), as_dp(ys))

    def free(self):
        if self.ptr:
            self._lib.lp_problem_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


@dataclass
class SolveOutput:
    result: dict
    trace: np.ndarray = field(default_factory=lambda: np.zeros((0, TRACE_WIDTH)))
    info: dict = field(default_factory=dict)


def make_options(precision: int = 0, max_refinements: int = 0, inner_eps: float = 0.0) -> Options:
    o = Options()
    o.precision, o.max_refinements, o.inner_eps = precision, max_refinements, inner_eps
    return o


def solve(problem: Problem, params: PdhgParameters | None = None, trace_cap: int = 0,
          library: C.CDLL | None = None, precision: int = PRECISION_FP64,
          max_refinements: int = 0) -> SolveOutput:
    """Solve through pdlp_solve_ex (FP64) or pdlp_solve_opts (FP32 +
    refinement); raises on failure."""
    L = library or lib()
    if precision != PRECISION_FP64:
        info = SolveInfo()
        o = make_options(precision, max_refinements)
        pp = C.byref(params) if params is not None else None
        r = L.pdlp_solve_opts(problem.ptr, pp, C.byref(o), C.byref(info))
        if not r:
            raise RuntimeError("solve failed: " + L.pdlp_last_error().decode())
        try:
            res = result_dict(r)
        finally:
            L.cupdlpx_result_free(r)
        return SolveOutput(res, np.zeros((0, TRACE_WIDTH)),
                           info_dict(info))
    tr = np.zeros((max(trace_cap, 1), TRACE_WIDTH))
    tl = C.c_int(0)
    info = SolveInfo()
    pp = C.byref(params) if params is not None else None
    r = L.pdlp_solve_ex(problem.ptr, pp, as_dp(tr) if trace_cap else None, trace_cap,
                        C.byref(tl), C.byref(info))
    if not r:
        raise RuntimeError("solve failed: " + L.pdlp_last_error().decode())
    try:
        res = result_dict(r)
    finally:
        L.cupdlpx_result_free(r)
    inf = info_dict(info)
    return SolveOutput(res, tr[: tl.value].copy(), inf)


class DeviceProblem:
    """An LP resident in HBM (pdlp_device_problem_t)."""

    def __init__(self, problem: Problem, library: C.CDLL | None = None):
        self._lib = library or lib()
        self.handle = self._lib.pdlp_device_problem_create(problem.ptr)
        if not self.handle:
            raise RuntimeError("upload failed: " + self._lib.pdlp_last_error().decode())

    @property
    def nbytes(self) -> int:
        return self._lib.pdlp_device_problem_bytes(self.handle)

    def solve(self, params: PdhgParameters | None = None, precision: int = PRECISION_FP64,
              max_refinements: int = 0) -> SolveOutput:
        info = SolveInfo()
        pp = C.byref(params) if params is not None else None
        o = make_options(precision, max_refinements)
        r = self._lib.pdlp_device_problem_solve_opts(self.handle, pp, C.byref(o), C.byref(info))
        if not r:
            raise RuntimeError("solve failed: " + self._lib.pdlp_last_error().decode())
        try:
            res = result_dict(r)
        finally:
            self._lib.cupdlpx_result_free(r)
        return SolveOutput(res, np.zeros((0, TRACE_WIDTH)),
                           info_dict(info))

    def time_kernels(self, params: PdhgParameters | None = None, reps: int = 20,
                     precision: int = PRECISION_FP64) -> np.ndarray:
        ms = np.zeros(4)
        pp = C.byref(params) if params is not None else None
        if self._lib.pdlp_device_problem_time_kernels_prec(self.handle, pp, precision, reps,
                                                           as_dp(ms)) != 0:
            raise RuntimeError("kernel timing failed: " + self._lib.pdlp_last_error().decode())
        return ms

    def free(self):
        if self.handle:
            self._lib.pdlp_device_problem_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Request loop over independent LPs (pdlp_server_t): `workers` threads,
    each with its own CUDA stream, admitting LPs by device-memory budget."""

    def __init__(self, params: PdhgParameters | None = None, precision: int = PRECISION_FP64,
                 workers: int = 8, mem_budget_bytes: int = 0, library: C.CDLL | None = None):
        self._lib = library or lib()
        o = make_options(precision)
        pp = C.byref(params) if params is not None else None
        self.handle = self._lib.pdlp_server_create(pp, C.byref(o), workers, mem_budget_bytes)
        if not self.handle:
            raise RuntimeError("server creation failed: " + self._lib.pdlp_last_error().decode())

    def submit(self, problem: Problem) -> int:
        """Request id, or -2 when the queue bound refused the request."""
        rid = self._lib.pdlp_server_submit(self.handle, problem.ptr)
        if rid == -2:
            return -2
        if rid < 0:
            raise RuntimeError("submit failed")
        return rid

    def set_queue_limit(self, host_bytes: int) -> None:
        if self._lib.pdlp_server_set_queue_limit(self.handle, host_bytes) != 0:
            raise ValueError("bad queue limit")

    def submit_bytes(self, payload: bytes) -> int:
        rid = self._lib.pdlp_server_submit_bytes(self.handle, payload, len(payload))
        if rid < 0:
            raise RuntimeError("submit failed: malformed payload")
        return rid

    def wait(self, rid: int) -> tuple[dict, dict]:
        info = RequestInfo()
        r = self._lib.pdlp_server_wait(self.handle, rid, C.byref(info))
        if not r:
            raise RuntimeError("request failed: " + self._lib.pdlp_last_error().decode())
        try:
            res = result_dict(r)
        finally:
            self._lib.cupdlpx_result_free(r)
        return res, {f: getattr(info, f) for f, _ in RequestInfo._fields_}

    def stats(self) -> dict:
        st = ServerStats()
        self._lib.pdlp_server_stats(self.handle, C.byref(st))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            self._lib.pdlp_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_solve(problems: list, params: PdhgParameters | None = None,
                precision: int = PRECISION_FP64, workers: int = 8, mem_budget_bytes: int = 0,
                library: C.CDLL | None = None) -> tuple[list, dict]:
    """Solve independent LPs side by side (pdlp_batch_solve); returns the
    result dicts in input order and the batch statistics."""
    L = library or lib()
    n = len(problems)
    arr = (C.POINTER(LpProblem) * n)(*[p.ptr for p in problems])
    res = (C.POINTER(Result) * n)()
    info = BatchInfo()
    o = make_options(precision)
    pp = C.byref(params) if params is not None else None
    rc = L.pdlp_batch_solve(arr, n, pp, C.byref(o), workers, mem_budget_bytes, res,
                            C.byref(info))
    out = []
    for i in range(n):
        if res[i]:
            out.append(result_dict(res[i]))
            L.cupdlpx_result_free(res[i])
        else:
            out.append(None)
    if rc not in (0, -3):
        raise RuntimeError("batch failed: " + L.pdlp_last_error().decode())
    return out, {f: getattr(info, f) for f, _ in BatchInfo._fields_}
