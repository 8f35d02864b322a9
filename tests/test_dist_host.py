"""Multi-process host logic of bench.py on CPU (gloo, world size 2): the
whole-job rate takes the slowest rank's time (max over ranks) and counts the
units of every rank; the reference arm runs on rank 0 only."""
import json
import os
import socket
import sys

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    rate, t = bench.job_throughput(1.0 + rank, 100, ws)
    q.put((rank, rate, t))
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_is_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, t in res:
        assert t == 2.0            # the slowest rank
        assert rate == 2 * 100 / 2.0


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_throughput(0.5, 10, 1) == (20.0, 0.5)


def test_reference_arm_runs_on_rank_0_only():
    sys.path.insert(0, ROOT)
    import bench
    args = bench.parse([])
    assert bench.run_reference(args, 2, 1, 1) is None


def test_reference_arm_line_keeps_the_contract():
    """The reference arm end to end on the host cores at a small size (J <= 8):
    one JSON-ready dict with the keys the bench contract names."""
    sys.path.insert(0, ROOT)
    import bench
    args = bench.parse(["--impl", "reference", "--steps", "2", "--warmup", "3", "--jmax", "8", "--nvec", "256"])
    out = bench.run_reference(args, 1, 0, 0)
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in out, key
    assert out["impl"] == "reference" and out["value"] > 0 and out["warmup"] == 3 and out["steps"] == 2
    assert out["e2e"]["value"] == out["value"]
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
    assert out["cpu_baseline"]["kind"] == "port" and out["cpu_baseline"]["cores"] >= 1
    # every spawned process ran its BLAS with one thread (one process per core)
    assert out["cpu_baseline"]["threads_per_process"] == ["1"]
    json.dumps(out)


def test_bench_defaults_keep_the_timing_rules():
    """With no flags: one GPU, at least 3 warm-up steps, a bounded number of
    timed steps (50 steps of about 26 ms: the timed work stays near a second)."""
    sys.path.insert(0, ROOT)
    import bench
    args = bench.parse([])
    assert args.gpus == 1 and args.impl == "ours"
    assert args.warmup >= 3 and 1 <= args.steps <= 200
