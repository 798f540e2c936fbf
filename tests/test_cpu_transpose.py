"""The host transpose (pdlp_host_transpose) -- the order the upload path's
device transpose reproduces -- against SciPy's CSR -> CSC conversion, a
stable counting sort: bit-identical outputs, below and above the size at
which the transpose runs on several threads."""
import numpy as np
import pytest

import cupdlpx as cp


def _csr(rng, m, n, mean_per_row):
    lengths = rng.poisson(mean_per_row, size=m)
    rows = np.repeat(np.arange(m), lengths)
    cols = rng.integers(0, n, size=rows.size)
    order = np.lexsort((cols, rows))
    ptr = np.zeros(m + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    return ptr, cols[order].astype(np.int32), rng.standard_normal(rows.size)


@pytest.mark.parametrize("m,n,per_row", [(500, 800, 6), (3000, 40, 9),
                                         (200_000, 300_000, 21)])  # 4.2M: threaded
def test_host_transpose_matches_stable_csc(lib, m, n, per_row):
    sp = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(3)
    ptr, col, val = _csr(rng, m, n, per_row)
    ref = sp.csr_matrix((val, col, ptr), shape=(m, n)).tocsc()
    tp = np.zeros(n + 1, dtype=np.int32)
    tj = np.zeros(len(val), dtype=np.int32)
    tx = np.zeros(len(val))
    assert lib.pdlp_host_transpose(m, n, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val),
                                   cp.as_ip(tp), cp.as_ip(tj), cp.as_dp(tx)) == 0
    assert np.array_equal(tp, ref.indptr)
    assert np.array_equal(tj, ref.indices)
    assert np.array_equal(tx.view(np.int64), ref.data.view(np.int64))


def test_host_transpose_rejects_bad_columns(lib):
    ptr = np.array([0, 2], dtype=np.int32)
    col = np.array([0, 3], dtype=np.int32)  # 3 >= n
    val = np.ones(2)
    tp, tj, tx = np.zeros(4, dtype=np.int32), np.zeros(2, dtype=np.int32), np.zeros(2)
    assert lib.pdlp_host_transpose(1, 3, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val),
                                   cp.as_ip(tp), cp.as_ip(tj), cp.as_dp(tx)) == -1


def test_host_transpose_rejects_malformed_row_pointers(lib):
    col = np.array([0, 1], dtype=np.int32)
    val = np.ones(2)
    tp, tj, tx = np.zeros(3, dtype=np.int32), np.zeros(2, dtype=np.int32), np.zeros(2)
    for ptr in ([0, 2, 1], [1, 1, 2]):  # decreasing; not starting at 0
        p = np.array(ptr, dtype=np.int32)
        assert lib.pdlp_host_transpose(2, 2, cp.as_ip(p), cp.as_ip(col), cp.as_dp(val),
                                       cp.as_ip(tp), cp.as_ip(tj), cp.as_dp(tx)) == -1
