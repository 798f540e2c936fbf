"""The SpMV plan (pdlp_spmv_plan): the tiling the kernels trust for every
shared-memory index.  Checked on CPU over random and adversarial row-length
distributions: every row in exactly one block, in order; light tiles within
TILE non-zeros and 1,024 rows; long rows only in chunks of at most the chunk
length, contiguous and in order; the register-path choice by its rule."""
import numpy as np
import pytest

import cupdlpx as cp

MAX_ROWS = 1024
MIN_AVG = 16


def _plan(lib, lengths, tile, chunk=0):
    ptr = np.zeros(len(lengths) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    nblk, nlong, direct = (np.zeros(1, dtype=np.int32) for _ in range(3))
    assert lib.pdlp_spmv_plan(len(lengths), cp.as_ip(ptr), tile, chunk, None, 0, cp.as_ip(nblk),
                              cp.as_ip(nlong), cp.as_ip(direct)) == 0
    blocks = np.zeros((max(int(nblk[0]), 1), 4), dtype=np.int32)
    assert lib.pdlp_spmv_plan(len(lengths), cp.as_ip(ptr), tile, chunk, cp.as_ip(blocks),
                              int(nblk[0]), cp.as_ip(nblk), cp.as_ip(nlong),
                              cp.as_ip(direct)) == 0
    return ptr, blocks[:int(nblk[0])], int(nlong[0]), int(direct[0])


def _check(ptr, blocks, nlong, direct, tile, chunk):
    rows = len(ptr) - 1
    nnz = int(ptr[-1])
    r = 0
    lid = 0
    qualifying = 0
    i = 0
    while i < len(blocks):
        x, y, z, w = (int(v) for v in blocks[i])
        assert x == r, "blocks cover the rows in order"
        if y >= 0:  # light tile of whole rows
            R, L = y - x, w - z
            assert 1 <= R <= MAX_ROWS
            assert z == ptr[x] and w == ptr[y]
            assert 0 <= L <= tile
            assert all(ptr[j + 1] - ptr[j] <= tile for j in range(x, y))
            if R > 1 and L <= 64 * R and L >= MIN_AVG * R:
                qualifying += L
            r = y
            i += 1
        else:  # chunks of one long row, in order
            assert -y - 1 == lid
            length = int(ptr[x + 1] - ptr[x])
            assert length > tile
            nch = -(-length // chunk)
            pos = int(ptr[x])
            for c in range(nch):
                cx, cy, cz, cw = (int(v) for v in blocks[i + c])
                assert (cx, cy, cz) == (x, y, pos)
                assert 0 < cw - cz <= chunk
                pos = cw
            assert pos == ptr[x + 1]
            lid += 1
            r = x + 1
            i += nch
    assert r == rows and lid == nlong
    want = int(tile == 1024 and nnz > 0 and 2 * qualifying >= nnz)
    assert direct == want


def _shapes(rng):
    yield "poisson20", rng.poisson(20, size=30000)
    yield "ones_and_twos", rng.integers(1, 3, size=50000)
    yield "empty_heavy", np.where(rng.random(40000) < 0.8, 0, rng.integers(1, 30, size=40000))
    yield "zipf", np.minimum(50000, (rng.pareto(1.2, size=20000) * 2).astype(int) + 1)
    yield "edges", np.array([511, 512, 513, 1023, 1024, 1025, 2047, 2048, 2049, 8192, 8193,
                             16384, 16385, 0, 0, 1, 100000])
    yield "all_empty", np.zeros(5000, dtype=int)
    yield "single_long", np.array([123457])


@pytest.mark.parametrize("tile", [512, 1024, 2048])
def test_plan_tiles_stay_within_the_kernel_bounds(lib, tile):
    rng = np.random.default_rng(17)
    for name, lengths in _shapes(rng):
        for chunk in (0, tile, 2 * tile):
            ptr, blocks, nlong, direct = _plan(lib, lengths, tile, chunk)
            eff = chunk if chunk else min(8 * tile, 8192)
            _check(ptr, blocks, nlong, direct, tile, eff)


def test_register_path_choice_by_row_shape(lib):
    rng = np.random.default_rng(5)
    assert _plan(lib, rng.poisson(20, size=20000), 1024)[3] == 1   # rows of ~20
    assert _plan(lib, rng.poisson(20, size=20000), 512)[3] == 0    # tiles of 512
    assert _plan(lib, rng.integers(1, 5, size=20000), 1024)[3] == 0  # rows of 1-4
    assert _plan(lib, np.array([30000, 40000]), 1024)[3] == 0       # long rows only


def test_plan_rejects_malformed_row_pointers(lib):
    ptr = np.array([0, 5, 3], dtype=np.int32)
    out = np.zeros(1, dtype=np.int32)
    assert lib.pdlp_spmv_plan(2, cp.as_ip(ptr), 1024, 0, None, 0, cp.as_ip(out), cp.as_ip(out),
                              cp.as_ip(out)) == -1
    good = np.array([0, 1], dtype=np.int32)
    assert lib.pdlp_spmv_plan(1, cp.as_ip(good), 1000, 0, None, 0, cp.as_ip(out), cp.as_ip(out),
                              cp.as_ip(out)) == -1
