"""pdlp_spmv_noalloc: the SpMV entry point that allocates no device memory.

It serves callers that cannot let a library call cudaMalloc -- an
application whose pool allocator already owns the GPU's memory, or a
latency-critical loop that must not take the synchronisation an allocation
implies.  The caller passes device buffers; the kernel's scratch is a fixed
array inside the library.  These checks call it through the C ABI on buffers
the test owns and compare it with the plan-based pdlp_gpu_spmv and with the
CPU oracle's SpMV, on two different matrices in a row (so that the second
call runs over scratch the first one left behind), and once more to see the
shared scratch give the same bits again.  Malformed matrices (a column out
of range, decreasing row pointers) are flagged on the device -- the kernel
reads such entries as zero and never dereferences them -- and the next valid
call must clear that flag and succeed.

The file name sorts last so that a run stopping at the first failure has run
every other test before this one.
"""
import ctypes as C

import numpy as np
import pytest

import cupdlpx as cp

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _bind(lib):
    lib.pdlp_spmv_noalloc.restype = C.c_int
    lib.pdlp_spmv_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.pdlp_spmv_noalloc_error.restype = C.c_char_p
    lib.pdlp_spmv_noalloc_error.argtypes = []


def _matrix(rng, lengths, cols):
    ptr = np.zeros(len(lengths) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    col = np.concatenate([np.sort(rng.choice(cols, size=L, replace=False)) if L else
                          np.zeros(0, dtype=np.int64) for L in lengths]).astype(np.int32)
    return ptr, col, rng.standard_normal(int(ptr[-1]))


def _plan_spmv(lib, ptr, col, val, x):
    rows = len(ptr) - 1
    y = np.zeros(rows)
    rc = lib.pdlp_gpu_spmv(rows, len(x), cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val),
                           cp.as_dp(x), cp.as_dp(y), 2048)
    assert rc == 0
    return y


def _oracle_spmv(oracle, ptr, col, val, x):
    y = np.zeros(len(ptr) - 1)
    oracle.oracle_spmv(len(ptr) - 1, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val), cp.as_dp(x),
                       cp.as_dp(y), 0)
    return y


def _noalloc_call(lib, ptr, col, val, x, nnz=None):
    """(return code, y) of one call on device copies of the arrays."""
    dev = torch.device("cuda:0")
    d_ptr = torch.from_numpy(ptr).to(dev)
    d_col = torch.from_numpy(col).to(dev)
    d_val = torch.from_numpy(val).to(dev)
    d_x = torch.from_numpy(x).to(dev)
    d_y = torch.full((len(ptr) - 1,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    rc = lib.pdlp_spmv_noalloc(len(ptr) - 1, len(x), int(ptr[-1] if nnz is None else nnz),
                               d_ptr.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                               d_x.data_ptr(), d_y.data_ptr(), C.c_void_p(stream.cuda_stream))
    return rc, d_y.cpu().numpy()


def _noalloc_spmv(lib, ptr, col, val, x):
    rc, y = _noalloc_call(lib, ptr, col, val, x)
    assert rc == 0, lib.pdlp_spmv_noalloc_error()
    return y


def _tolerance(ptr, col, val, x):
    # both products differ from the exact sum by at most n u sum|a x| per row
    rows = len(ptr) - 1
    absum = np.zeros(rows)
    np.add.at(absum, np.repeat(np.arange(rows), np.diff(ptr)), np.abs(val * x[col]))
    return 2 * 1.2e-16 * np.maximum(np.diff(ptr), 1) * absum


def test_noalloc_spmv_matches_plan_spmv_twice(lib, oracle):
    _bind(lib)
    rng = np.random.default_rng(5)
    cols = 40000
    # first: power-law rows, several running across many 2048-non-zero tiles
    first = np.minimum(cols, (rng.pareto(1.1, size=3000) * 4).astype(int) + 1)
    first[[10, 11, 500]] = [9000, 2048, 30000]
    # second: fewer, shorter rows with empty ones, so fewer tiles than before
    second = np.where(rng.random(4000) < 0.3, 0, rng.integers(1, 25, size=4000))
    second[-1] = 5000
    results = []
    for lengths in (first, second):
        ptr, col, val = _matrix(rng, lengths, cols)
        x = rng.standard_normal(cols)
        y_ref = _plan_spmv(lib, ptr, col, val, x)
        y_cpu = _oracle_spmv(oracle, ptr, col, val, x)
        y = _noalloc_spmv(lib, ptr, col, val, x)
        assert np.all(np.isfinite(y))
        tol = _tolerance(ptr, col, val, x)
        assert np.all(np.abs(y - y_ref) <= tol)
        assert np.all(np.abs(y - y_cpu) <= tol)
        results.append((ptr, col, val, x, y))
    # the first matrix again, over the scratch the second call left: same bits
    ptr, col, val, x, y = results[0]
    assert np.array_equal(_noalloc_spmv(lib, ptr, col, val, x), y)


def test_noalloc_spmv_rejects_sizes_above_limit(lib):
    _bind(lib)
    ptr = np.array([0, 1], dtype=np.int32)
    over = 65536 * 2048 + 1  # PDLP_NOALLOC_MAX_TILES tiles of 2048 non-zeros, plus one
    # rejected on the host before any device buffer is touched
    rc = lib.pdlp_spmv_noalloc(1, 1, over, ptr.ctypes.data, None, None, None, None, None)
    assert rc == -3
    assert b"exceeds" in lib.pdlp_spmv_noalloc_error()


def test_noalloc_spmv_flags_malformed_csr_then_recovers(lib, oracle):
    _bind(lib)
    cols = 6
    x = np.arange(1.0, cols + 1.0)
    good_ptr = np.array([0, 2, 3, 5], dtype=np.int32)
    good_col = np.array([0, 4, 2, 1, 5], dtype=np.int32)
    val = np.array([1.0, -2.0, 0.5, 3.0, 4.0])
    # a column index past the last column: read as zero, flagged
    bad_col = good_col.copy()
    bad_col[1] = cols + 7
    rc, _ = _noalloc_call(lib, good_ptr, bad_col, val, x)
    assert rc == -4
    assert b"column index out of range" in lib.pdlp_spmv_noalloc_error()
    # row pointers that decrease (row 1 would end before it starts): skipped, flagged
    bad_ptr = np.array([0, 3, 1, 5], dtype=np.int32)
    rc, _ = _noalloc_call(lib, bad_ptr, good_col, val, x)
    assert rc == -4
    assert b"malformed row pointers" in lib.pdlp_spmv_noalloc_error()
    # the flag starts at zero again: the next valid call succeeds, exactly
    y = _noalloc_spmv(lib, good_ptr, good_col, val, x)
    np.testing.assert_array_equal(y, _oracle_spmv(oracle, good_ptr, good_col, val, x))
