"""The C ABI without a GPU: exports, struct layouts, host-side errors.

- every function declared in include/*.h is exported by the library;
- the ctypes mirror in cupdlpx.py has the C layout of include/cupdlpx_types.h,
  and that layout equals the reference's own include/cupdlpx_types.h where
  the reference sources are present (compiled with gcc, offsetof/sizeof);
- loading fails loudly when the CUDA library is missing (no CPU fallback);
- host-side argument checks reject bad input before any CUDA call.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
REF_INCLUDE = os.path.join(oracle_lib.reference_dir(), "include")
SHIM = os.path.join(ROOT, "oracle", "ref_shim")

STRUCTS = {"LpProblem": "lp_problem_t", "RestartParameters": "restart_parameters_t",
           "TerminationCriteria": "termination_criteria_t", "GridSize": "grid_size_t",
           "PdhgParameters": "pdhg_parameters_t", "Result": "cupdlpx_result_t",
           "MatrixDesc": "matrix_desc_t"}
# this library's own structures (include/pdlp_gb300.h)
EXT_STRUCTS = {"SolveInfo": "pdlp_solve_info_t", "Options": "pdlp_options_t",
               "RequestInfo": "pdlp_request_info_t", "ServerStats": "pdlp_server_stats_t",
               "BatchInfo": "pdlp_batch_info_t"}


def declared_functions():
    names = set()
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        text = "\n".join(l for l in text.splitlines() if not l.lstrip().startswith("#"))
        for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(([^;{}()]*)\)\s*;", text):
            if m.group(1) not in ("if", "while", "for", "return", "sizeof"):
                names.add(m.group(1))
    return sorted(names)


def test_headers_declare_the_reference_api():
    names = declared_functions()
    for f in ("create_lp_problem", "set_start_values", "solve_lp_problem",
              "set_default_parameters", "cupdlpx_result_free", "lp_problem_free"):
        assert f in names


@pytest.mark.parametrize("name", declared_functions())
def test_library_exports_every_declared_function(lib, name):
    assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def _layout_program(tmp_path, structs, header):
    lines = ["#include <stddef.h>", "#include <stdio.h>", f'#include "{header}"',
             "int main(void) {"]
    for py, ct in structs.items():
        lines.append(f'  printf("{py} . %zu %zu\\n", sizeof({ct}), _Alignof({ct}));')
        for f, _t in getattr(cp, py)._fields_:
            lines.append(f'  printf("{py} {f} %zu %zu\\n", offsetof({ct}, {f}), '
                         f'sizeof((({ct} *)0)->{f}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    return src


def _c_layout(tmp_path, incs, tag, structs=STRUCTS, header="cupdlpx_types.h"):
    src = _layout_program(tmp_path, structs, header)
    exe = tmp_path / f"layout_{tag}"
    r = subprocess.run(["gcc", "-std=gnu11", *[f"-I{i}" for i in incs], str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return {(a, b): (int(c), int(d)) for a, b, c, d in (l.split() for l in out.splitlines())}


def _ctypes_layout(structs=STRUCTS):
    lay = {}
    for py in structs:
        S = getattr(cp, py)
        lay[(py, ".")] = (C.sizeof(S), C.alignment(S))
        for f, t in S._fields_:
            lay[(py, f)] = (getattr(S, f).offset, C.sizeof(t))
    return lay


def test_ctypes_mirror_matches_c_header_layout(tmp_path):
    assert _c_layout(tmp_path, [INCLUDE], "ours") == _ctypes_layout()
    assert _c_layout(tmp_path, [INCLUDE], "ext", EXT_STRUCTS, "pdlp_gb300.h") == \
        _ctypes_layout(EXT_STRUCTS)


def test_header_layout_matches_reference_header(tmp_path):
    if not os.path.exists(os.path.join(REF_INCLUDE, "cupdlpx_types.h")):
        pytest.skip("reference sources not present on this host")
    ours = _c_layout(tmp_path, [INCLUDE], "ours")
    theirs = _c_layout(tmp_path, [SHIM, REF_INCLUDE], "ref")
    assert ours == theirs


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(cp, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(cp, "_LIB", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        cp.lib()


def test_create_lp_problem_rejects_unsupported_format(lib):
    d = cp.MatrixDesc()
    d.m, d.n, d.fmt = 2, 2, 9
    c = np.zeros(2)
    assert not lib.create_lp_problem(cp.as_dp(c), C.byref(d), None, None, None, None, None)
    assert lib.pdlp_last_error()


def test_create_lp_problem_copies_and_fills_defaults(lib):
    # NULL objective -> 0, NULL bounds -> -inf / +inf (reference src/cupdlpx.c:105-114)
    prob = cp.Problem.from_csr([0, 1, 2], [0, 1], [2.0, 3.0], 2, library=lib)
    a = prob.arrays()
    assert np.array_equal(a["c"], [0.0, 0.0])
    assert np.all(a["lv"] == -np.inf) and np.all(a["uv"] == np.inf)
    assert np.all(a["lc"] == -np.inf) and np.all(a["uc"] == np.inf)
    assert a["c0"] == 0.0


def test_set_start_values_replaces_previous_start(lib):
    prob = cp.Problem.from_csr([0, 1], [0], [1.0], 1, library=lib)
    prob.set_start(x=np.array([1.0]), y=np.array([2.0]))
    prob.set_start(x=np.array([3.0]))
    s = prob.ptr.contents
    assert s.primal_start[0] == 3.0
    assert not s.dual_start


def test_noalloc_spmv_host_checks_need_no_gpu(lib):
    lib.pdlp_spmv_noalloc.restype = C.c_int
    lib.pdlp_spmv_noalloc.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6
    # above the fixed scratch: rejected before any CUDA call
    assert lib.pdlp_spmv_noalloc(1, 1, 65536 * 2048 + 1, None, None, None, None, None, None) == -3
    assert lib.pdlp_spmv_noalloc(-1, 1, 1, None, None, None, None, None, None) == -1
    assert lib.pdlp_spmv_noalloc(0, 5, 0, None, None, None, None, None, None) == 0
    # non-zeros without rows is an inconsistent CSR, rejected before any CUDA call
    assert lib.pdlp_spmv_noalloc(0, 5, 3, None, None, None, None, None, None) == -1


def test_generators_are_deterministic(lib):
    for kind, args in (("random", (300, 700, 3000, 4)), ("powerlaw", (500, 900, 6000, 1.2, 50, 2)),
                       ("transport", (5, 7, 3))):
        a = cp.Problem.generated(kind, *args, library=lib).arrays()
        b = cp.Problem.generated(kind, *args, library=lib).arrays()
        for k in ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv"):
            assert np.array_equal(a[k], b[k]), (kind, k)
        # CSR well formed: sorted, distinct columns in every row
        rp, cj = a["row_ptr"], a["col_ind"]
        assert rp[0] == 0 and rp[-1] == len(cj) and np.all(np.diff(rp) >= 0)
        for r in range(a["m"]):
            row = cj[rp[r]:rp[r + 1]]
            assert np.all(np.diff(row) > 0)


def test_create_rejects_malformed_csc_and_coo(lib):
    """CSC and COO inputs are converted on the host; a column pointer that is
    not monotone or disagrees with the declared non-zeros, and indices
    outside the matrix, give NULL instead of reads or writes out of bounds."""
    c = np.zeros(3)
    rows = np.array([0, 1, 1], dtype=np.int32)
    cols = np.array([0, 2, 1], dtype=np.int32)
    vals = np.ones(3)
    for col_ptr, nnz in (([0, 2, 1, 3], 3), ([0, 1, 2, 3], 2), ([1, 1, 2, 3], 3)):
        ptr = np.array(col_ptr, dtype=np.int32)
        d = cp.MatrixDesc()
        d.m, d.n, d.fmt, d.zero_tolerance = 2, 3, cp.MATRIX_CSC, 0.0
        d.data.csc.nnz = nnz
        d.data.csc.col_ptr, d.data.csc.row_ind, d.data.csc.vals = (
            cp.as_ip(ptr), cp.as_ip(rows), cp.as_dp(vals))
        assert not lib.create_lp_problem(cp.as_dp(c), C.byref(d), None, None, None, None, None)
    for r, k in (([0, 2, 1], [0, 1, 2]), ([0, 1, 1], [0, 3, 1]), ([-1, 0, 1], [0, 1, 2])):
        rr, kk = np.array(r, dtype=np.int32), np.array(k, dtype=np.int32)
        d = cp.MatrixDesc()
        d.m, d.n, d.fmt, d.zero_tolerance = 2, 3, cp.MATRIX_COO, 0.0
        d.data.coo.nnz = 3
        d.data.coo.row_ind, d.data.coo.col_ind, d.data.coo.vals = (
            cp.as_ip(rr), cp.as_ip(kk), cp.as_dp(vals))
        assert not lib.create_lp_problem(cp.as_dp(c), C.byref(d), None, None, None, None, None)
