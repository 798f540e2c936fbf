"""bench.py host logic on CPU: algorithmic byte counts, replica device
selection, the max-over-ranks reduction on a two-rank gloo group, and the
reference arm's JSON line on the small seeded LP."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_kernel_bytes_at_the_powerlaw_lp():
    m, n, nnz = 1_000_000, 2_000_000, 20_000_000
    primal, dual = bench.kernel_bytes(m, n, nnz, 8)
    # A^T stream + row pointers + gathered y + 7 n-vectors; A stream + pointers + x + 5 m-vectors
    assert primal == 12 * nnz + 4 * (n + 1) + 8 * m + 56 * n
    assert dual == 12 * nnz + 4 * (m + 1) + 8 * n + 40 * m
    assert primal + dual == 668_000_008
    p32, d32 = bench.kernel_bytes(m, n, nnz, 4)
    assert primal - p32 == 4 * nnz + 4 * m + 28 * n


def test_visible_device_for_rank():
    assert bench.visible_device_for_rank(0, None) == "0"
    assert bench.visible_device_for_rank(3, None) == "3"
    assert bench.visible_device_for_rank(1, "4,6") == "6"


def test_max_over_ranks_without_process_group():
    assert bench.max_over_ranks([1.5, 2.0]) == [1.5, 2.0]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench as b
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        q.put((rank, b.max_over_ranks([float(rank + 1), 10.0 - rank])))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: [2.0, 10.0], 1: [2.0, 10.0]}


def test_reference_arm_prints_one_json_line(lib, oracle):
    env = dict(os.environ, PDLP_QUIET="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "random_m2k_n5k_nnz20k_seed0", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    # without a GPU the FP64 oracle stands in for the reference's own GPU solve
    assert d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["config"]["workload"] == "random_m2k_n5k_nnz20k_seed0"
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
