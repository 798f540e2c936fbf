"""The upload path's device transpose (pdlp_gpu_transpose: a stable radix
sort of the column indices on the GPU) against the host transpose and SciPy's
stable CSR -> CSC conversion: bit-identical row pointers, column indices and
values, on random, power-law, duplicate-entry and edge-case matrices."""
import numpy as np
import pytest

import cupdlpx as cp

pytestmark = pytest.mark.gpu


def _transpose(fn, m, n, ptr, col, val):
    tp = np.zeros(n + 1, dtype=np.int32)
    tj = np.zeros(max(len(val), 1), dtype=np.int32)
    tx = np.zeros(max(len(val), 1))
    assert fn(m, n, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val), cp.as_ip(tp), cp.as_ip(tj),
              cp.as_dp(tx)) == 0
    return tp, tj[:len(val)], tx[:len(val)]


def _check(lib, m, n, ptr, col, val):
    g = _transpose(lib.pdlp_gpu_transpose, m, n, ptr, col, val)
    h = _transpose(lib.pdlp_host_transpose, m, n, ptr, col, val)
    assert np.array_equal(g[0], h[0])
    assert np.array_equal(g[1], h[1])
    assert np.array_equal(g[2].view(np.int64), h[2].view(np.int64))
    return g


def _csr(rng, m, n, lengths):
    rows = np.repeat(np.arange(m), lengths)
    cols = rng.integers(0, n, size=rows.size)
    order = np.lexsort((cols, rows))
    ptr = np.zeros(m + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    return ptr, cols[order].astype(np.int32), rng.standard_normal(rows.size)


@pytest.mark.parametrize("m,n,per_row", [(500, 800, 6), (3000, 40, 9), (70_000, 300, 3),
                                         (200_000, 3_000_000, 21)])
def test_gpu_transpose_matches_host_and_scipy(lib, m, n, per_row):
    rng = np.random.default_rng(11)
    ptr, col, val = _csr(rng, m, n, rng.poisson(per_row, size=m))
    tp, tj, tx = _check(lib, m, n, ptr, col, val)
    sp = pytest.importorskip("scipy.sparse")
    ref = sp.csr_matrix((val, col, ptr), shape=(m, n)).tocsc()
    assert np.array_equal(tp, ref.indptr) and np.array_equal(tj, ref.indices)


def test_gpu_transpose_powerlaw_lp(lib):
    # the column-degree mix of the power-law benchmark LP (1-entry columns up
    # to 50,000-entry ones), at a twentieth of its size
    p = cp.Problem.generated("powerlaw", 50000, 100000, 1000000, 1.2, 50000, 1)
    a = p.arrays()
    _check(lib, a["m"], a["n"], a["row_ptr"], a["col_ind"], a["vals"])


def test_gpu_transpose_edge_cases(lib):
    rng = np.random.default_rng(5)
    # duplicate entries within rows keep their input order
    ptr = np.array([0, 4, 4, 7], dtype=np.int32)
    col = np.array([2, 2, 0, 2, 1, 1, 2], dtype=np.int32)
    _check(lib, 3, 4, ptr, col, np.arange(1.0, 8.0))
    # no non-zeros; one column; empty rows and columns
    _check(lib, 5, 3, np.zeros(6, dtype=np.int32), np.zeros(0, dtype=np.int32), np.zeros(0))
    ptr, col, val = _csr(rng, 400, 1, rng.poisson(2, size=400))
    _check(lib, 400, 1, ptr, col, val)
    lengths = np.where(rng.random(1000) < 0.5, 0, rng.integers(1, 5, size=1000))
    ptr, col, val = _csr(rng, 1000, 70000, lengths)
    _check(lib, 1000, 70000, ptr, col, val)
