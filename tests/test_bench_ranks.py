"""The N > 1 path of bench.py on the CPU: world-size-2 gloo process groups.

Replicas only: each rank solves its own copy of the city, so the only
cross-rank step is the aggregation of the timed figures (slowest rank's
time, all ranks' cell-steps).  The reference arm runs on rank 0 alone.
"""

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r timed 100 + 25 r ms for 1e6 (r + 1) cell-steps
        q.put((rank, bench.aggregate_ranks(100.0 + 25.0 * rank, 1.0e6 * (rank + 1))))
    finally:
        dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        total_ms, cell_steps = out[r]
        assert total_ms == 125.0  # the slowest rank
        assert cell_steps == 3.0e6  # every rank's work


def test_aggregate_single_process_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.aggregate_ranks(12.5, 7.0) == (12.5, 7.0)


@pytest.mark.parametrize("rank", [1])
def test_reference_arm_runs_on_rank_zero_only(rank):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_json_line():
    """The reference arm's one JSON line: the oracle port on the host cores,
    with the keys the measurement contract names."""

    import json

    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--cpu-seconds", "1", "--mid-run-step", "3"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "cell-steps/s" and line["value"] > 0
    assert line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the same workload object as the GPU arm's line; the sample continues a run
    sys.path.insert(0, str(ROOT))
    import bench

    assert line["config"] == bench.workload_config(1)
    assert "continued from step 3 " in cb["sample"]
