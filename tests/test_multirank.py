"""The bench's multi-rank plumbing on the CPU: world_size-2 gloo ranks on 127.0.0.1 (the path the
GPU runs take under torchrun with one replica per GPU): the barrier and the max over ranks of the
timed region."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, td = bench.dist_init()
    try:
        bench.barrier(td)
        out.put((r, w, bench.allmax(td, 1.5 + r)))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 2.5), (1, 2, 2.5)]


def test_reference_arm_line():
    """`bench.py --impl reference` (one timed FP64 oracle solve of the 130,662-DOF shell on the host
    threads) prints one JSON line with the contract's keys and a converged solve."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       cwd=root, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "coupled residual" in d["cpu_baseline"]["sample"]
    res = float(d["cpu_baseline"]["sample"].split("to a ")[1].split(" coupled")[0])
    assert res < 1e-8
