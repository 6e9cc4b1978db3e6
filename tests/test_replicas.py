"""Host logic of the benchmark on CPU: the multi-process replica path (gloo, world size 2) with rank
discovery from the launcher's environment, the barrier, the maximum over ranks behind the whole-job
rate and the reference arm that only rank 0 runs; and the CPU baseline's record."""
import argparse
import contextlib
import io
import os
import socket
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def replica(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, REPO)
    import bench

    assert bench.dist_env() == (rank, world, rank)
    dist = bench.dist_init(world)
    try:
        # each rank processed 64 scans; rank r took 0.5 + 0.25 r seconds: the job took the slowest
        rate = bench.replica_rate(dist, world, 64, 0.5 + 0.25 * rank)
        slowest = 0.5 + 0.25 * (world - 1)
        assert abs(rate - world * 64 / slowest) < 1e-9, rate
        assert bench.dist_max(dist, float(10 - rank)) == 10.0
        bench.barrier(dist)
        # the reference arm: ranks other than 0 return at once without output
        if rank != 0:
            buf = io.StringIO()
            with contextlib.redirect_stdout(buf):
                bench.run_reference_arm(argparse.Namespace(scans=64, steps=1, warmup=0, gpus=world), rank, world)
            assert buf.getvalue() == ""
        bench.barrier(dist)
        with open(os.path.join(out_dir, f"rank{rank}.ok"), "w") as f:
            f.write(f"{rate:.6f}\n")
    finally:
        dist.destroy_process_group()


def test_replica_aggregate_gloo_world2(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.spawn(replica, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True)
    rates = [open(tmp_path / f"rank{r}.ok").read().strip() for r in range(world)]
    assert rates == [f"{world * 64 / 0.75:.6f}"] * world


def test_single_process_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench

    assert bench.dist_init(1) is None
    assert bench.replica_rate(None, 1, 64, 0.5) == 128.0
    bench.barrier(None)


def test_cpu_baseline_record(built):
    """The CPU baseline's record: the oracle over a bounded sample, the thread count it used."""
    sys.path.insert(0, REPO)
    import bench
    import lp_testlib as T

    cb = bench.cpu_baseline([T.synth_scan(1, 0)], budget_s=0.2, threads=1)
    assert cb["kind"] == "port" and cb["unit"] == "scans/s" and cb["cores"] == 1
    assert cb["value"] > 0 and "1 threads" in cb["sample"]
