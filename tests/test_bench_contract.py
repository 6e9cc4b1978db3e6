"""bench.py's JSON line on CPU: main() run against stand-ins for the device objects (context,
prepared batch, the shared library's page-locked allocator and lp_process_batch) carries every key
of the benchmark contract with consistent values, and a failing optional leg is reported in the
line instead of losing it."""
import contextlib
import ctypes
import io
import json
import sys

import numpy as np

import lp_testlib as T
from test_host_marshalling import PinningLibrary

lp = T.lp


class FakeContext:
    handle = None

    def __init__(self, device=0):
        self.device = device
        self.table = None

    def set_tuning_table(self, table):
        self.table = table

    def close(self):
        pass


TUNED = {"parts": 2, "balance_parts": 1, "hull_cta_min": 256, "hull_ctas_per_sm": 2, "cell_ctas_per_sm": 8,
         "jcp_ctas_per_sm": 8}


class FakeTuning:
    def __init__(self, d):
        self.d = dict(d)

    def as_dict(self):
        return dict(self.d)


class FakeKey:
    def as_tuple(self):
        return (1, 1, 1)


def fake_autotune(ctx, xs, pipe, cfgs, rings, iters=3, table=None):
    return FakeTuning(TUNED), {"trials": 14, "start_ms": 2.7, "best_ms": 2.5, "candidates": []}


class FakeResult:
    def __init__(self, n):
        self.n_obstacles = n // 2
        self.n_clusters = 3
        self.cluster_labels = np.full(n, -1, np.int32)
        self.cluster_labels[: n // 4] = 0
        self.hull_indices = np.arange(9, dtype=np.int32)


class FakeBatch:
    def __init__(self, ctx, xs, pipe, cfgs, rings):
        self.xs = xs
        self.tuning = FakeTuning(TUNED if ctx.table is not None else {})

    def execute(self):
        pass

    def synchronize(self):
        pass

    def capture_graph(self):
        pass

    def close(self):
        pass

    def download(self):
        return [FakeResult(len(x)) for x in self.xs]

    def profile(self):
        return [("k_bin", 0.05), ("k_scan", 0.01), ("k_jcp_rows", 0.40), ("k_hull", 0.30), ("k_scan", 0.01)]

    def time(self, iters, flush_l2=False):
        return 2.5


def run_main(monkeypatch, lib, argv):
    sys.path.insert(0, T.REPO)
    import bench

    monkeypatch.setattr(lp, "library", lambda: lib)
    monkeypatch.setattr(lp, "Context", FakeContext)
    monkeypatch.setattr(lp, "PreparedBatch", FakeBatch)
    monkeypatch.setattr(lp, "autotune", fake_autotune)
    monkeypatch.setattr(lp, "TuningTable", lambda: object())
    monkeypatch.setattr(lp, "tuning_key", lambda xs, cfgs: FakeKey())
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.main()
    return json.loads(out.getvalue().strip().splitlines()[-1])


def test_bench_line_carries_the_contract(monkeypatch):
    line = run_main(monkeypatch, PinningLibrary(), ["--steps", "3", "--warmup", "3", "--scans", "4", "--no-cpu",
                                                    "--no-serve", "--no-dror"])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "e2e", "gpu_launches", "roofline", "clocks", "cpu_baseline"):
        assert key in line, key
    assert line["n_gpus"] == 1 and line["steps"] == 3 and line["warmup"] == 3
    assert line["higher_is_better"] is True and line["scaling"] == "weak" and line["vs_baseline"] is None
    assert abs(line["value"] - 4 * 3 / (3 * 2.5e-3)) < 1e-6  # scans over the summed event time
    assert abs(line["ms_per_step"] - 2.5) < 1e-9
    assert line["config"]["workload"] == "batch4_mixed"
    # the autotuner ran first and the timed batch took its choice
    a = line["autotune"]
    assert a["chosen"] == TUNED and a["bucket"] == [1, 1, 1] and a["trials"] == 14
    assert a["tuned_ms"] <= a["default_ms"] and line["config"]["tuning"] == TUNED
    e = line["e2e"]
    assert e["unit"] == "scans/s" and e["value"] > 0 and e["h2d_bytes_per_step"] > 0 and e["d2h_bytes_per_step"] > 0
    # the stand-in profile has four of our kernels; k_scan counts three launches (tile sums, look-back, apply)
    assert line["gpu_launches"] == (3 + 3 * 2) * 3
    r = line["roofline"]
    assert r["kernel"] == "k_jcp_rows" and r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-12
    assert r["traffic"] is not None  # read from the ncu summary under profiles/
    assert set(line["clocks"]) >= {"sm_mhz", "sm_max_mhz", "reasons"}
    assert line["plain"]["scans"] == 4
    st = r["stage"]  # segmentation stage: k_bin, the prefix scan after it and k_jcp_rows in the stand-in profile
    assert abs(st["ms"] - 0.46) < 1e-12 and st["algorithmic_bytes"] == 20 * sum(len(x) for x in bench_points())
    assert abs(st["frac"] - st["achieved"] / r["peak"]) < 1e-12


def bench_points():
    import bench
    return [d[0] for d in bench.make_workload(4)]


def test_serving_and_outlier_sub_records(monkeypatch):
    """The default line carries the serving and outlier-filter sub-records as their legs return
    them; a failing leg is reported in its sub-record."""
    sys.path.insert(0, T.REPO)
    import bench

    monkeypatch.setattr(bench, "serve_leg", lambda duration: {"latency_ms": {"p99": 2.0}, "duration_s": duration})

    def broken(steps, warmup):
        raise RuntimeError("stand-in outlier failure")

    monkeypatch.setattr(bench, "dror_leg", broken)
    line = run_main(monkeypatch, PinningLibrary(), ["--steps", "3", "--warmup", "3", "--scans", "4", "--no-cpu",
                                                    "--no-plain"])
    assert line["serve"] == {"latency_ms": {"p99": 2.0}, "duration_s": 52.0}
    assert line["dror"] == {"error": "RuntimeError: stand-in outlier failure"}


class FailingLibrary(PinningLibrary):
    def lp_process_batch(self, *a):
        raise RuntimeError("stand-in failure")


def test_failed_end_to_end_leg_is_reported(monkeypatch):
    line = run_main(monkeypatch, FailingLibrary(), ["--steps", "3", "--warmup", "3", "--scans", "4", "--no-cpu",
                                                    "--no-plain", "--no-serve", "--no-dror"])
    assert line["e2e"] == {"error": "RuntimeError: stand-in failure", "unit": "scans/s"}
    assert line["value"] > 0 and line["plain"] is None
    assert ctypes.sizeof(lp.ScanOutput) > 0


def test_reference_arm_line(monkeypatch):
    """--impl reference on rank 0: the CPU baseline's rate as the line's value, its record (with the
    single-thread leg) under cpu_baseline, and an e2e entry with no host-device bytes."""
    sys.path.insert(0, T.REPO)
    import bench

    calls = []

    def fake_baseline(data, budget_s=20.0, threads=None):
        calls.append((len(data), budget_s, threads))
        return {"value": 70.0 if threads is None else 25.0, "unit": "scans/s", "cores": threads or 16,
                "kind": "port", "sample": "stand-in"}

    monkeypatch.setattr(bench, "cpu_baseline", fake_baseline)
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--steps", "4", "--warmup", "3", "--scans", "2"])
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.main()
    line = json.loads(out.getvalue().strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] == 70.0 and line["unit"] == "scans/s"
    assert line["metric"] == bench.METRIC and line["higher_is_better"] is True
    assert line["cpu_baseline"]["single_thread"]["cores"] == 1
    assert line["e2e"] == {"value": 70.0, "unit": "scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert calls == [(2, 20.0, None), (2, 20.0, 1)]
    assert line["config"]["workload"] == "batch2_mixed" and line["config"]["points"] > 0
