"""The multi-GPU mode of the benchmark is N independent replicas (the path
is not partitioned across GPUs): each rank times its own problem, the step
time is the max over ranks, and the throughput counts every rank's dofs.
That bookkeeping runs here on two gloo ranks on the CPU."""

import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        R = bench.Replicas(world, "cpu")
        R.barrier()
        ms = 10.0 + 5.0 * rank  # rank 1 is the slower replica
        dofs = 1000.0 * (rank + 1)  # replicas may differ in size
        ms_max = R.max(ms)
        total = R.total(dofs)
        q.put((rank, ms_max, total, R.gdofs_per_s(total, ms_max)))
        R.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_time_and_total_dofs():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms_max, total, value in out:
        assert ms_max == 15.0
        assert total == 3000.0
        assert abs(value - 3000.0 / 15e-3 / 1e9) < 1e-18


def test_single_replica_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    R = bench.Replicas(1, "cpu")
    R.barrier()
    assert R.max(7.0) == 7.0 and R.total(5.0) == 5.0


def test_bench_defaults_and_host_helpers(monkeypatch):
    """bench.py's defaults keep the run contract (1 GPU, at least 3 warm-up
    steps, our implementation), and its host helpers read the committed
    profile summary and the peak file."""
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert a.gpus == 1 and a.impl == "ours" and a.warmup >= 3 and a.steps >= 1
    cfg = bench.workload_config(a, 2146689, 60859905)
    assert cfg["cells"] == 6 * 64 ** 3 and cfg["dofs"] == 2146689 and cfg["nnz"] == 60859905
    assert cfg["parallelism"] == "single"
    peak, kind = bench.measured_peaks()
    assert peak > 0 and kind in ("measured", "fallback")
    assert bench.profile_traffic("sell_f32_p2_64") == 399360512
    assert bench.profile_traffic("no such kernel") is None


def test_reference_arm_times_full_steps(monkeypatch, capsys):
    """bench.py --impl reference runs W + K full steps of the oracle on the
    host threads and prints one JSON line whose timed region is the steps
    it ran (no extrapolation)."""
    import json

    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--n", "4",
                                      "--steps", "2", "--warmup", "1"])
    bench.run_reference(bench.parse())
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and "full step" in cpu["sample"]
    assert len(cpu["cg_iterations"]) == 2 and min(cpu["cg_iterations"]) > 0
    assert line["ms_per_step"] * 1e-3 * 2 <= line["wall_s"]
