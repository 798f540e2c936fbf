"""Kernel-level parity on the GPU: fused SpMV, GPU rescaling, power method,
each against the CPU oracle on the same seeded inputs."""
import ctypes as C

import numpy as np
import pytest

import cupdlpx as cp
import oracle_lib as ol

pytestmark = pytest.mark.gpu


def _csr_with_shapes(rng, rows, cols, lengths):
    ptr = np.zeros(rows + 1, dtype=np.int32)
    ptr[1:] = np.cumsum(lengths)
    nnz = int(ptr[-1])
    col = np.concatenate([np.sort(rng.choice(cols, size=L, replace=False)) if L else
                          np.zeros(0, dtype=np.int64) for L in lengths]).astype(np.int32)
    val = rng.standard_normal(nnz)
    return ptr, col, val


# (tile, kernel variant): staged tiles of 512, 1024 and 2048 non-zeros; the
# register path for short-row tiles (1024), also on column and value arrays
# off 16-byte boundaries (scalar loads)
KERNELS = [(512, 0), (2048, 0), (1024, 0), (1024, 1), (1024, 2)]


@pytest.mark.parametrize("tile,variant", KERNELS)
@pytest.mark.parametrize("shape", ["short", "mixed", "long", "empty_rows", "single", "rows20"])
def test_spmv_matches_oracle(lib, oracle, tile, variant, shape):
    rng = np.random.default_rng(11)
    cols = 60000
    if shape == "short":
        lengths = rng.integers(0, 12, size=3000)
    elif shape == "rows20":  # rows of ~20 non-zeros: every tile on the register path
        lengths = rng.poisson(20, size=4000)
    elif shape == "mixed":  # power-law rows: most light, some longer than a tile
        lengths = np.minimum(cols, (rng.pareto(1.1, size=2500) * 3).astype(int) + 1)
    elif shape == "long":
        lengths = np.array([5000, 2048, 2049, 1, 7000, 0, 513])
    elif shape == "empty_rows":
        lengths = np.where(rng.random(5000) < 0.7, 0, rng.integers(1, 40, size=5000))
    else:
        lengths = np.array([30000])
    ptr, col, val = _csr_with_shapes(rng, len(lengths), cols, lengths)
    x = rng.standard_normal(cols)
    y = np.zeros(len(lengths))
    rc = lib.pdlp_gpu_spmv_variant(len(lengths), cols, cp.as_ip(ptr), cp.as_ip(col),
                                   cp.as_dp(val), cp.as_dp(x), cp.as_dp(y), tile, variant)
    assert rc == 0
    yo = np.zeros(len(lengths))
    oracle.oracle_spmv(len(lengths), cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val), cp.as_dp(x),
                       cp.as_dp(yo), 1)
    # summation-order differences only: |y - yo| <= 2 n u sum|a x| per row
    absum = np.zeros(len(lengths))
    np.add.at(absum, np.repeat(np.arange(len(lengths)), np.diff(ptr)), np.abs(val * x[col]))
    tol = 2 * 1.2e-16 * np.maximum(np.diff(ptr), 1) * absum
    assert np.all(np.abs(y - yo) <= tol)
    # bitwise reproducible run to run
    y2 = np.zeros_like(y)
    lib.pdlp_gpu_spmv_variant(len(lengths), cols, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val),
                              cp.as_dp(x), cp.as_dp(y2), tile, variant)
    assert np.array_equal(y, y2)


def test_spmv_register_path_matches_staged_bitwise_on_aligned_and_offset_arrays(lib):
    # the vector-load and scalar-load forms of the register path sum in the
    # same order
    rng = np.random.default_rng(5)
    lengths = rng.poisson(20, size=3000)
    ptr, col, val = _csr_with_shapes(rng, len(lengths), 50000, lengths)
    x = rng.standard_normal(50000)
    ys = []
    for variant in (1, 2):
        y = np.zeros(len(lengths))
        assert lib.pdlp_gpu_spmv_variant(len(lengths), 50000, cp.as_ip(ptr), cp.as_ip(col),
                                         cp.as_dp(val), cp.as_dp(x), cp.as_dp(y), 1024,
                                         variant) == 0
        ys.append(y)
    assert np.array_equal(ys[0], ys[1])


def test_spmv_variant_rejects_register_path_off_tile_1024(lib):
    ptr = np.array([0, 1], dtype=np.int32)
    col = np.array([0], dtype=np.int32)
    val, x, y = np.ones(1), np.ones(1), np.zeros(1)
    for tile, variant in ((512, 1), (2048, 2), (1024, 3), (1000, 0)):
        assert lib.pdlp_gpu_spmv_variant(1, 1, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val),
                                         cp.as_dp(x), cp.as_dp(y), tile, variant) != 0


def test_spmv_rejects_bad_columns(lib):
    ptr = np.array([0, 2], dtype=np.int32)
    col = np.array([0, 5], dtype=np.int32)  # 5 >= cols
    val = np.ones(2)
    x = np.ones(3)
    y = np.zeros(1)
    assert lib.pdlp_gpu_spmv(1, 3, cp.as_ip(ptr), cp.as_ip(col), cp.as_dp(val), cp.as_dp(x),
                             cp.as_dp(y), 512) != 0


def _gpu_rescale(lib, prob, params):
    a = prob.arrays()
    m, n, nnz = a["m"], a["n"], a["nnz"]
    out = {k: np.zeros(s) for k, s in (("vals", nnz), ("c", n), ("lv", n), ("uv", n),
                                       ("lc", m), ("uc", m), ("con", m), ("var", n))}
    cb, ob = C.c_double(), C.c_double()
    rc = lib.pdlp_gpu_rescale(prob.ptr, C.byref(params), *[cp.as_dp(out[k]) for k in
                              ("vals", "c", "lv", "uv", "lc", "uc", "con", "var")],
                              C.byref(cb), C.byref(ob))
    assert rc == 0, lib.pdlp_last_error()
    out["cb"], out["ob"] = cb.value, ob.value
    return out


@pytest.mark.parametrize("ruiz,pc,alpha,bo", [(10, True, 1.0, True), (0, True, 1.0, True),
                                              (4, False, 1.0, False), (10, True, 0.5, True)])
def test_gpu_rescale_matches_oracle(lib, oracle, ruiz, pc, alpha, bo):
    prob = cp.Problem.generated("random", 700, 1500, 9000, 3)
    p = ol.oracle_params(oracle)
    p.l_inf_ruiz_iterations, p.has_pock_chambolle_alpha = ruiz, pc
    p.pock_chambolle_alpha, p.bound_objective_rescaling = alpha, bo
    g = _gpu_rescale(lib, prob, p)
    o = ol.oracle_rescale(oracle, prob, p)
    # Ruiz maxima, sqrt, divisions and the sequential PC sums are exact
    # restatements: the scaled matrix and the cumulative scalings are
    # bit-identical (alpha = 1; general alpha goes through pow()).
    exact = alpha == 1.0
    for k in ("vals", "con", "var"):
        if exact:
            assert np.array_equal(g[k], o[k]), k
        else:
            np.testing.assert_allclose(g[k], o[k], rtol=1e-13)
    # bound/objective norms are tree sums on the GPU: scalars to 1e-15
    assert abs(g["cb"] - o["cb"]) <= 1e-15 * o["cb"]
    assert abs(g["ob"] - o["ob"]) <= 1e-15 * o["ob"]
    for k in ("c", "lv", "uv", "lc", "uc"):
        np.testing.assert_allclose(g[k], o[k], rtol=1e-14, atol=0)


def test_power_method_matches_oracle(lib, oracle):
    prob = cp.Problem.generated("random", 800, 2000, 12000, 5)
    p = ol.oracle_params(oracle)
    s, it = C.c_double(), C.c_int()
    assert lib.pdlp_gpu_power_method(prob.ptr, C.byref(p), C.byref(s), C.byref(it)) == 0
    # oracle on the oracle-scaled matrix from the same mt19937(1) start
    o = ol.oracle_rescale(oracle, prob, p)
    a = prob.arrays()
    v0 = np.zeros(a["m"])
    oracle.oracle_power_start_vector(a["m"], cp.as_dp(v0))
    oit = C.c_int()
    so = oracle.oracle_power_method(a["m"], a["n"], cp.as_ip(a["row_ptr"]), cp.as_ip(a["col_ind"]),
                                    cp.as_dp(o["vals"]), cp.as_dp(v0), p.sv_max_iter, p.sv_tol,
                                    C.byref(oit), 0)
    assert abs(it.value - oit.value) <= 1
    assert abs(s.value - so) <= 1e-9 * so
