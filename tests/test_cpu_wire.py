"""Binary problem format (the reference's serialize_lp_problem_to_ptr layout,
src/distribution_utils.cu:279-405) on CPU: the byte image written field by
field with struct, round trips, and rejection of truncated or inconsistent
payloads."""
import struct

import numpy as np
import pytest

import cupdlpx as cp


def _expected_bytes(a, ps=None, ds=None):
    n, m, nnz = a["n"], a["m"], a["nnz"]
    out = struct.pack("<iiid", n, m, nnz, a["c0"])
    for k in ("c", "lv", "uv", "lc", "uc"):
        out += a[k].astype("<f8").tobytes()
    out += a["row_ptr"].astype("<i4").tobytes() + a["col_ind"].astype("<i4").tobytes()
    out += a["vals"].astype("<f8").tobytes()
    out += struct.pack("<ii", ps is not None, ds is not None)
    if ps is not None:
        out += np.asarray(ps, "<f8").tobytes()
    if ds is not None:
        out += np.asarray(ds, "<f8").tobytes()
    return out


def test_layout_matches_the_reference_format(lib):
    prob = cp.Problem.generated("random", 40, 90, 300, 3, library=lib)
    a = prob.arrays()
    data = prob.to_bytes()
    assert data == _expected_bytes(a)
    assert lib.pdlp_problem_wire_size(prob.ptr) == len(data)
    # with start values
    xs, ys = np.linspace(0, 1, a["n"]), np.linspace(-1, 1, a["m"])
    prob.set_start(x=xs, y=ys)
    assert prob.to_bytes() == _expected_bytes(a, xs, ys)


def test_round_trip(lib):
    prob = cp.Problem.from_csr([0, 2, 3], [0, 2, 1], [1.5, -2.0, 3.0], 3, c=[1.0, 0.0, -1.0],
                               lc=[-np.inf, 1.0], uc=[4.0, np.inf], lv=[0, -1, -np.inf],
                               uv=[np.inf, 2, 5], c0=7.25, library=lib)
    prob.set_start(y=np.array([0.5, -0.5]))
    back = cp.Problem.from_bytes(prob.to_bytes(), library=lib)
    a, b = prob.arrays(), back.arrays()
    for k in ("row_ptr", "col_ind", "vals", "c", "lc", "uc", "lv", "uv"):
        assert np.array_equal(a[k], b[k]), k
    assert b["c0"] == 7.25
    s = back.ptr.contents
    assert not s.primal_start and s.dual_start[1] == -0.5
    assert back.to_bytes() == prob.to_bytes()


def test_rejects_truncated_and_inconsistent_payloads(lib):
    prob = cp.Problem.generated("random", 20, 50, 120, 9, library=lib)
    data = prob.to_bytes()
    for cut in (0, 5, 12, 20, len(data) // 2, len(data) - 1):
        with pytest.raises(ValueError):
            cp.Problem.from_bytes(data[:cut], library=lib)
    bad = bytearray(data)
    # a column index past n
    a = prob.arrays()
    off = 20 + 8 * (3 * a["n"] + 2 * a["m"]) + 4 * (a["m"] + 1)
    bad[off:off + 4] = struct.pack("<i", a["n"] + 5)
    with pytest.raises(ValueError):
        cp.Problem.from_bytes(bytes(bad), library=lib)
    # a negative size
    with pytest.raises(ValueError):
        cp.Problem.from_bytes(struct.pack("<iiid", -1, 0, 0, 0.0) + b"\0" * 8, library=lib)


def test_rejects_payloads_with_hostile_counts(lib):
    # sizes near INT_MAX must be rejected by the length checks, never read
    big = 2**31 - 1
    for n, m, nnz in ((big, 0, 0), (0, big, 0), (0, 0, big), (big, big, big), (1, big, 1)):
        head = struct.pack("<iiid", n, m, nnz, 0.0)
        for tail in (b"", b"\0" * 64):
            with pytest.raises(ValueError):
                cp.Problem.from_bytes(head + tail, library=lib)
    # random counts over a valid payload's bytes
    prob = cp.Problem.generated("random", 20, 50, 120, 9, library=lib)
    data = bytearray(prob.to_bytes())
    rng = np.random.default_rng(0)
    for _ in range(200):
        bad = bytearray(data)
        bad[:12] = struct.pack("<iii", *rng.integers(-5, 400, size=3))
        try:
            cp.Problem.from_bytes(bytes(bad), library=lib)
        except ValueError:
            pass
