"""bench.py's multi-rank logic on CPU: gloo, world size 2.

Under torchrun every rank runs its own replica of the problem (the path has
no cross-rank exchange), the job is timed by the slowest rank, and the rate
is weak-scaling: world x steps / max time.  The reference arm runs on rank 0
only; the other ranks exit 0 without output.
"""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    ms = [12.5, 20.0][rank]
    mx = bench.max_over_ranks(ms, world)
    rate = bench.whole_job_rate(10, mx, world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, mx, rate))


def test_max_over_ranks_and_weak_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, rate in out:
        assert mx == 20.0
        assert rate == pytest.approx(2 * 10 / 0.020)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, 1) == 7.0
    assert bench.whole_job_rate(4, 8.0, 1) == pytest.approx(500.0)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_prints_the_contract_line():
    """Rank 0 of the reference arm times the CPU restatement on a small sample
    of the workload (the first points of the same data, the same initial
    state) and prints one JSON line with the metric, unit and config of the
    GPU arm, its cpu_baseline (flagged as extrapolated, with the three CPU
    variants) and a zero-copy e2e."""
    import json
    sys.path.insert(0, ROOT)
    import bench
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--ref-sample", "64"], env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["unit"] == "EM iters/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["N"] == 1_000_000 and d["config"]["K"] == 8000 and d["config"]["D"] == 166
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["extrapolated"] is True and cb["extrapolated"] is True and d["sample_points"] == 64
    assert set(cb["variants"]) == {"faithful", "port_omp", "blas"}
    assert cb["variants"]["faithful"]["cores"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": "EM iters/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
