"""The pipelined step kernel's tiling (pdlp_spmv_pipe_plan), the facts its
bulk copies and shared-memory indexing rely on, checked on CPU:

- tiles cover the rows once, in order; packed tiles hold 1..256 whole rows
  and at most 2,048 non-zeros, a row of more than 128 non-zeros is alone,
  a row of more than 2,048 is cut into ordered chunks of at most 2,048;
- in every precision the solver runs (8-byte values and vectors, 4-byte,
  4-byte values with 8-byte vectors) each copy range starts on a 16-byte
  boundary, is a multiple of 16 bytes, ends inside its array's allocation
  (256-byte aligned, padded to a multiple of 256 bytes), and the tile's
  ranges fit one stage buffer.
"""
import numpy as np
import pytest

import cupdlpx as cp


def _plan(lib, lengths, nv):
    ptr = np.zeros(len(lengths) + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    nt, nl = np.zeros(1, dtype=np.int32), np.zeros(1, dtype=np.int32)
    lim = np.zeros(4, dtype=np.int32)
    assert lib.pdlp_spmv_pipe_plan(len(lengths), cp.as_ip(ptr), nv, None, None, 0,
                                   cp.as_ip(nt), cp.as_ip(nl), cp.as_ip(lim)) == 0
    k = max(int(nt[0]), 1)
    tiles = np.zeros((k, 4), dtype=np.int32)
    nbytes = np.zeros(k, dtype=np.int32)
    assert lib.pdlp_spmv_pipe_plan(len(lengths), cp.as_ip(ptr), nv, cp.as_ip(tiles),
                                   cp.as_ip(nbytes), k, cp.as_ip(nt), cp.as_ip(nl), None) == 0
    return ptr, tiles[:int(nt[0])], nbytes[:int(nt[0])], int(nl[0]), lim


def _alloc_elems(count, size):
    # Arena::take: 256-byte aligned, count * size + 1 bytes rounded up to 256
    return ((count * size + 1 + 255) // 256 * 256) // size


def _ranges(tile, sm, st, nv):
    """(first element, element count, element size, array) of each copy."""
    r0, r1, k0, k1 = (int(v) for v in tile)
    out = []
    if r1 >= 0:
        a = r0 & ~3
        out.append((a, ((r1 + 1 + 3) & ~3) - a, 4, "ptr"))
        tv = 16 // st
        if r1 > r0:
            a = r0 & ~(tv - 1)
            for _ in range(nv):
                out.append((a, ((r1 + tv - 1) & ~(tv - 1)) - a, st, "vec"))
    if k1 > k0:
        a = k0 & ~3
        out.append((a, ((k1 + 3) & ~3) - a, 4, "col"))
        mv = 16 // sm
        a = k0 & ~(mv - 1)
        out.append((a, ((k1 + mv - 1) & ~(mv - 1)) - a, sm, "val"))
    return out


def _check(ptr, tiles, nbytes, nlong, lim, nv):
    rows_cap, tile_cap, med, stage = (int(v) for v in lim)
    rows, nnz = len(ptr) - 1, int(ptr[-1])
    r, i, lid = 0, 0, 0
    while i < len(tiles):
        x, y, z, w = (int(v) for v in tiles[i])
        assert x == r
        if y >= 0:
            R, L = y - x, w - z
            assert 1 <= R <= rows_cap and 0 <= L <= tile_cap
            assert z == ptr[x] and w == ptr[y]
            if R > 1:
                assert all(ptr[j + 1] - ptr[j] <= med for j in range(x, y))
            r, i = y, i + 1
        else:
            assert -y - 1 == lid
            length = int(ptr[x + 1] - ptr[x])
            assert length > tile_cap
            nch = -(-length // tile_cap)
            pos = int(ptr[x])
            for c in range(nch):
                cx, cy, cz, cw = (int(v) for v in tiles[i + c])
                assert (cx, cy, cz) == (x, y, pos) and 0 < cw - cz <= tile_cap
                pos = cw
            assert pos == ptr[x + 1]
            r, i, lid = x + 1, i + nch, lid + 1
    assert r == rows and lid == nlong
    n_arr = {"ptr": rows + 1, "vec": rows, "col": nnz, "val": nnz}
    for t, b in zip(tiles, nbytes):
        assert b <= stage
        for sm, st in ((8, 8), (4, 4), (4, 8)):
            total = 0
            for a, cnt, size, arr in _ranges(t, sm, st, nv):
                assert (a * size) % 16 == 0 and (cnt * size) % 16 == 0 and cnt > 0
                assert a + cnt <= _alloc_elems(n_arr[arr], size)
                total += cnt * size
            assert total <= b


SHAPES = {
    "ones": [1] * 3000,
    "empty_and_short": [0, 0, 3, 0, 1, 0, 0, 0, 2] * 400,
    "mixed": None,
    "long_rows": [5, 2049, 1, 0, 4097, 6000, 128, 129, 2048, 2047, 3],
    "all_empty": [0] * 700,
}


@pytest.mark.parametrize("name", sorted(SHAPES))
@pytest.mark.parametrize("nv", [4, 5])
def test_pipe_plan_invariants(lib, name, nv):
    lengths = SHAPES[name]
    if lengths is None:
        rng = np.random.default_rng(3)
        lengths = np.minimum(9000, (rng.pareto(1.2, size=20000) + 1).astype(int) - 1)
    _check(*_plan(lib, list(lengths), nv), nv)


@pytest.mark.parametrize("nv", [4, 5])
def test_pipe_plan_on_powerlaw_rows(lib, nv):
    # both matrices of a seeded power-law LP (rows of A ~ 20 non-zeros;
    # A^T: a Zipf column-degree mix of 1-non-zero rows and rows up to 50,000)
    p = cp.Problem.generated("powerlaw", 50000, 100000, 1000000, 1.2, 50000, 1)
    a = p.arrays()
    lenA = np.diff(a["row_ptr"])
    lenT = np.bincount(a["col_ind"], minlength=a["n"])
    for lengths in (lenA, lenT):
        _check(*_plan(lib, [int(v) for v in lengths], nv), nv)
