"""bench.py on the host: the reference arm's JSON line at a small size carries the keys the bench
contract names (also when launched on two ranks), the adjoint cost arithmetic (difference of two
run lengths) is right, and the replica aggregation of --gpus N (slowest rank's time, every rank's
cells) holds on two gloo ranks."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--size", "24,12,12",
                        "--steps", "4", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "MLUPS" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 4 and d["warmup"] == 3
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_adjoint_report_cancels_fixed_cost():
    sys.path.insert(0, str(ROOT))
    import bench
    plain = 0.02e-3                            # s per forward step
    fixed_f, fixed_b = 5e-3, 26e-3             # s per call
    per_f, per_b = 0.021e-3, 0.045e-3          # s per step
    t = {n: (fixed_f + per_f * n, fixed_b + per_b * n) for n in (2000, 1000)}
    rep = bench._adjoint_report({"steps": 2000, "half": 1000, "t": t}, plain)
    assert rep["backward_ms_per_step"] == pytest.approx(per_b * 1e3)
    assert rep["forward_ckpt_ms_per_step"] == pytest.approx(per_f * 1e3)
    assert rep["backward_over_forward"] == pytest.approx(per_b / plain)
    assert rep["backward_fixed_ms_per_call"] == pytest.approx(fixed_b * 1e3)
    assert rep["backward_call_over_forward"] == pytest.approx((fixed_b + per_b * 2000) / (2000 * plain))


def _replica_worker(rank, world, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sec = 0.5 + rank            # rank 1 is the slowest replica
        bench.replica_barrier(world)
        worst = bench.replica_max(sec, world)
        q.put((rank, worst, bench.replica_mlups(1000, 10, worst, world)))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_two_ranks_gloo():
    # bench.py --gpus N runs one independent domain per rank; the job's time is the slowest rank's
    # and the value counts every rank's cells (world_size 2 over gloo on the host)
    import multiprocessing as mp
    import socket
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [1.5, 1.5]
    assert all(o[2] == pytest.approx(2 * 1000 * 10 / 1.5 / 1e6) for o in out)


def test_reference_arm_under_torchrun_two_ranks():
    # the driver launches --impl reference like the GPU arm; rank 0 alone runs and prints
    import socket
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        port = sck.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
                        "--size", "16,8,8", "--steps", "2", "--warmup", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["impl"] == "reference"
