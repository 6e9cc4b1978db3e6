"""Benchmark of the per-scan perception path (segmentation -> clustering -> hull + OBB).

Workload "batch64_mixed": 64 seeded synthetic scans of uneven size in one launch sequence (ring
count {32,64,128}, azimuth bins {1024,2048,4096}, return rate U[0.3,1], 10-200 obstacles, flat /
sloped / undulating ground), ~8.3M float32 XYZI points; one step = the whole pipeline over the
batch. `value` is device-resident scans/s of the batched form (captured CUDA graph), `e2e` the same
metric through the C ABI with host buffers (H2D + D2H inside the timed region). The plain form (one
scan per launch sequence) is timed on the same scans for the batched/plain ratio, and the CPU
oracle (a restatement of the reference path) on a bounded sample of the same workload.

The line also carries a serving sub-record (six sensors at 10 Hz with bursts, >= 3,000 scans,
p50/p99/p99.9 latency) and an outlier-filter sub-record (32 x 1M-point scans, DROR stage roofline).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  small profiling case: python bench.py --steps 2 --warmup 1 --scans 16 --no-cpu --no-plain --no-e2e --no-serve --no-dror
Multi-GPU (torchrun): replicas, one independent batch per rank (scans do not shard a step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "lidar-processing-v2_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

WORKLOAD = 3
METRIC = "scans/s (batched, 64 mixed scans, exact labels)"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def dist_init(world):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def dist_max(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def replica_rate(dist, world, units, seconds):
    """Whole-job rate of N replicas: every rank processed `units` in its own `seconds`; the job
    takes as long as its slowest rank, so the aggregate is N x units over the maximum time."""
    return world * units / dist_max(dist, seconds)


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def workload_name(nscans):
    return "batch64_mixed" if nscans == 64 else f"batch{nscans}_mixed"


def make_workload(nscans):
    import lidar_gb300 as lp

    return [lp.synth_scan(WORKLOAD, i) for i in range(nscans)]


def cpu_baseline(data, budget_s=20.0, threads=None):
    """The oracle (CPU restatement of the reference path) over scans of the same workload, one
    scan per thread (the reference objects are not thread-safe, so each thread runs its own)."""
    import lp_testlib as T
    import lidar_gb300 as lp
    from concurrent.futures import ThreadPoolExecutor

    threads = threads or (os.cpu_count() or 1)
    pipe = lp.PipelineConfig.default()
    T.oracle()
    done = []
    t0 = time.perf_counter()

    def work(k):
        x, ring, cfg = data[k % len(data)]
        T.o_process(x, ring, cfg, pipe)
        return len(x)

    with ThreadPoolExecutor(max_workers=threads) as ex:
        k = 0
        while time.perf_counter() - t0 < budget_s and k < 4 * len(data):
            batch = list(range(k, k + threads))
            done += list(ex.map(work, batch))
            k += threads
    dt = time.perf_counter() - t0
    return {"value": len(done) / dt, "unit": "scans/s", "cores": threads, "kind": "port",
            "sample": f"{len(done)} scans of the batch64_mixed workload ({sum(done)} points) through the CPU oracle "
                      f"restatement of the reference path, {threads} threads, {dt:.1f} s"}


def e2e_leg(lp, ctx, pipe, xs, rings, cfgs, steps):
    """End to end through the C ABI with host buffers: the scans sit in page-locked host memory and
    every step copies them in, runs the whole path and copies every result back out into page-locked
    result buffers reused from step to step (as a sensor node reuses its messages; the call's
    argument structs are built once, as a C++ caller keeps its lp_scan_input array). Returns the
    mean seconds per step (the first step untimed) and the bytes copied in and out per step."""
    pin_x = [lp.pinned_copy(x) for x in xs]
    pin_r = [lp.pinned_copy(r) for r in rings]
    bufs = [lp.ResultBuffers(len(x), pinned=True) for x in xs]
    call = lp.BatchCall(pin_x, pipe, cfgs, pin_r, outputs=bufs)
    times = []
    for it in range(max(3, steps // 2) + 1):
        t1 = time.perf_counter()
        call.run(ctx)
        dt = time.perf_counter() - t1
        if it > 0:
            times.append(dt)
    h2d = sum(x.nbytes + r.nbytes for x, r in zip(pin_x, pin_r))
    # per scan: noise u8 + seg u32 + cluster i32 labels; hull offsets and indices; z range; two boxes
    d2h = sum(len(b.seg) * 9 + 4 * (b.out.n_clusters + 1 + b.out.n_hull_indices) + 8 * b.out.n_clusters
              + 2 * 72 * b.out.n_clusters for b in bufs)
    return float(np.mean(times)), int(h2d), int(d2h)


def leg_error(exc):
    return f"{type(exc).__name__}: {exc}"


def kernel_profile(batch):
    prof = batch.profile()
    agg = {}
    for name, ms in prof:
        a = agg.setdefault(name, [0, 0.0])
        a[0] += 1
        a[1] += ms
    return prof, agg


def run_reference_arm(args, rank, world):
    if rank != 0:
        return
    data = make_workload(args.scans)
    budget = max(10.0, min(120.0, 5.0 * args.steps))
    cb = cpu_baseline(data, budget_s=budget)
    # the reference's own design: one processor thread
    cb["single_thread"] = cpu_baseline(data, budget_s=min(budget, 20.0), threads=1)
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "scans/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(args.scans), "scans": args.scans,
                       "points": int(sum(len(d[0]) for d in data)), "generator_seed": "1000*3+scan"},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "scans/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def serve_leg(duration):
    """Serving workload: six sensors at 10 Hz (periods ~ N(100 ms, 10 ms)), the rate doubled
    during the first second of every 5 s, scans of 32/64/128 rings x 1024-4096 bins (synthetic
    workload 5), a 20 GB admission budget. Latency = submission -> results in host buffers.
    Returns the record (latency percentiles, rates, clocks)."""
    import lidar_gb300 as lp

    sensors, per_sensor = 6, 8
    pool = [[lp.synth_scan(5, s * per_sensor + k) for k in range(per_sensor)] for s in range(sensors)]
    pipe = lp.PipelineConfig.default()
    server = lp.Server(0, pipe, memory_budget_bytes=20 << 30, max_batch_scans=16, slots=3)
    rng = np.random.default_rng(5000)
    events = []
    for s in range(sensors):
        t = float(rng.uniform(0.0, 0.1))
        k = 0
        while t < duration:
            events.append((t, s, k))
            k += 1
            period = float(rng.normal(0.100, 0.010))
            if (t % 5.0) < 1.0:
                period *= 0.5
            t += max(period, 0.005)
    events.sort()
    done = {}
    stop = threading.Event()
    warm = sensors * per_sensor
    t_end = [time.perf_counter() + 1e9]

    def poller():
        while not stop.is_set() or len(done) < len(events) + warm:
            for d, _ in server.poll(wait_us=2000):
                done[int(d.tag)] = (d.latency_ms, d.queue_ms, d.batch_scans, d.status)
            if stop.is_set() and time.perf_counter() - t_end[0] > 30:
                break

    # warm-up: every pool scan once
    for s in range(sensors):
        for k in range(per_sensor):
            x, ring, cfg = pool[s][k]
            server.submit(x, ring, cfg, 1_000_000 + s * per_sensor + k)
    th = threading.Thread(target=poller, daemon=True)
    th.start()
    while sum(1 for t in list(done) if t >= 1_000_000) < warm:
        time.sleep(0.01)
    with ClockSampler(0) as clocks:
        t0 = time.perf_counter()
        for i, (t, s, k) in enumerate(events):
            dt = t0 + t - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            x, ring, cfg = pool[s][k % per_sensor]
            server.submit(x, ring, cfg, i)
        t_end[0] = time.perf_counter()
        stop.set()
        th.join(timeout=60)
    stats = server.stats()
    server.close()
    lat = np.array([done[i][0] for i in range(len(events)) if i in done])
    bs = np.array([done[i][2] for i in range(len(events)) if i in done])
    ok = sum(1 for i in range(len(events)) if i in done and done[i][3] == 0)
    pts = [len(pool[s][k % per_sensor][0]) for _, s, k in events]
    return {"workload": "serve_6x10Hz_mixed", "sensors": sensors, "duration_s": duration,
            "burst": "rate x2 during the first 1 s of every 5 s", "memory_budget_gb": 20,
            "scans": int(len(lat)), "ok": int(ok), "offered_scans_per_s": len(events) / duration,
            "achieved_scans_per_s": len(lat) / max(t_end[0] - t0, 1e-9),
            "points_per_scan": {"min": int(min(pts)), "max": int(max(pts)), "mean": float(np.mean(pts))},
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "p99.9": float(np.percentile(lat, 99.9)), "max": float(lat.max())},
            "batch_scans": {"mean": float(bs.mean()), "max": int(bs.max())},
            "server": stats, "clocks": clocks.summary()}


def run_serve(args):
    r = serve_leg(args.duration)
    line = {"metric": "serving latency p99 ms/scan (6 sensors x 10 Hz, continuous batching)",
            "value": r["latency_ms"]["p99"], "unit": "ms", "higher_is_better": False, "n_gpus": 1,
            "data": "synthetic", "dtype": "f32", "config": {"workload": r["workload"]}, **r}
    print(json.dumps(line))


def dror_leg(steps, warmup, distinct=4, ns=32):
    """Outlier-filter workload: 32 unorganised scans of 1.0 M points (128-ring geometry at 16384
    bins, 950k returns + 50k clutter within 15 m, shuffled; synthetic workload 4) per launch. DROR
    with multiplier 3 x 0.17 deg (rad), min neighbours 3, min radius 0.1 m on the input (the
    reference's kd-tree search replayed), then the unorganised segmentation, clustering and hulls.
    `distinct` generated scans are repeated to `ns` (32 in the workload; fewer for a profiling case).
    Returns the record (stage time, roofline)."""
    import lidar_gb300 as lp

    uniq = [lp.synth_scan(4, i) for i in range(min(distinct, ns))]
    data = [uniq[i % len(uniq)] for i in range(ns)]
    xs = [d[0] for d in data]
    cfgs = []
    for d in data:
        c = d[2]
        c.assume_unorganized_cloud = 1
        cfgs.append(c)
    noise = lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180.0, 0.1, 3)
    pipe = lp.PipelineConfig.default(enable_noise_removal=1, noise=noise)
    ctx = lp.Context(0)
    npts = sum(len(x) for x in xs)
    batch = lp.PreparedBatch(ctx, xs, pipe, cfgs, None)
    batch.execute()
    batch.synchronize()
    res = batch.download()
    noise_pts = int(sum(int(r.noise_labels.sum()) for r in res))
    _, agg = kernel_profile(batch)
    dror_kernels = [k for k in agg if k.startswith("k_kt_")]
    dror_ms = sum(agg[k][1] for k in dror_kernels)
    total_ms = sum(a[1] for a in agg.values())
    batch.capture_graph()
    for _ in range(warmup):
        batch.execute()
    batch.synchronize()
    with ClockSampler(0) as clocks:
        step_ms = [batch.time(1, flush_l2=False) for _ in range(steps)]
    ms = float(np.mean(step_ms))
    peak, peak_kind = measured_peaks()
    if not dror_ms > 0:
        raise RuntimeError("no outlier-filter kernel in the batch profile")
    dror_gbs = 17.0 * npts / (dror_ms / 1e3) / 1e9
    top = max(agg.items(), key=lambda kv: kv[1][1])
    batch.close()
    ctx.close()
    return {"workload": f"dror{ns}x1M", "scans": ns, "distinct_scans": len(uniq), "points": npts,
            "dror": "multiplier 3*0.17deg, min_neighbours 3, min radius 0.1 m; the reference kd-tree search",
            "scans_per_s": ns / (ms / 1e3), "ms_per_step": ms, "points_per_s": npts / (ms / 1e3),
            "noise_points": noise_pts,
            "dror_stage": {"ms": dror_ms, "kernels": {k: round(agg[k][1], 3) for k in dror_kernels},
                           "points_per_s": npts / (dror_ms / 1e3), "share_of_step": dror_ms / total_ms,
                           "roofline": {"bound": "hbm", "achieved": dror_gbs, "peak": peak, "unit": "GB/s",
                                        "frac": dror_gbs / peak, "algorithmic_bytes_per_point": 17,
                                        "peak_source": peak_kind}},
            "top_kernel": {"name": top[0], "share": top[1][1] / total_ms},
            "clocks": clocks.summary()}


def run_dror(args):
    r = dror_leg(args.steps, args.warmup, args.dror_unique, args.dror_scans)
    line = {"metric": f"scans/s ({args.dror_scans} x 1.0M-point unorganised scans, DROR + pipeline)", "value": r["scans_per_s"],
            "unit": "scans/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "dtype": "f32", "data": "synthetic", "config": {"workload": r["workload"]}, **r}
    print(json.dumps(line))


# Kernels of the segmentation stage (ring partition, polar grid, RECM, RANSAC, projection, dilation,
# jump convolution, label write-back); prefix scans count with the stage of the kernel before them.
SEG_KERNELS = {"k_quadrant", "k_ring_count", "k_ring_apply", "k_bin", "k_scatter", "k_cell_small", "k_cell_large",
               "k_chain", "k_near", "k_ransac_draw", "k_ransac_inliers", "k_ransac_select", "k_label_depth",
               "k_project_key", "k_pixel", "k_dilate_rows", "k_jcp_weights", "k_jcp_rowrec", "k_jcp_rows",
               "k_populate"}


def stage_ms(prof, kernels):
    """Summed event time of the named kernels and of the prefix scans launched right after them."""
    tot, prev = 0.0, None
    for name, ms in prof:
        if name == "k_scan":
            if prev in kernels:
                tot += ms
            continue
        prev = name
        if name in kernels:
            tot += ms
    return tot


def traffic_bytes(kernel, alg_bytes):
    """DRAM bytes per launch of `kernel`: the measured ratio of DRAM traffic (dram__bytes_read.sum +
    dram__bytes_write.sum from one ncu capture, summarised under profiles/) to the launch's
    algorithmic bytes, times this launch's algorithmic bytes; None without a capture."""
    import glob
    for path in glob.glob(os.path.join(REPO, "profiles", "*.md")):
        for line in open(path):
            f = line.split()
            if len(f) == 3 and f[0] == "traffic_ratio" and f[1] == kernel:
                return int(float(f[2]) * alg_bytes)
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--serve", action="store_true", help="multi-sensor serving workload instead of the batch bench")
    ap.add_argument("--dror", action="store_true", help="32 x 1M-point outlier-filter workload")
    ap.add_argument("--dror-unique", type=int, default=4, help="distinct generated scans in --dror (repeated)")
    ap.add_argument("--dror-scans", type=int, default=32, help="scans per batch in --dror (32 for the workload)")
    ap.add_argument("--duration", type=float, default=60.0, help="seconds of simulated sensor stream (--serve)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--scans", type=int, default=64, help="scans per batch (64 for the headline workload)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--no-plain", action="store_true", help="skip the one-scan-per-launch form")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end run")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving sub-record")
    ap.add_argument("--no-dror", action="store_true", help="skip the outlier-filter sub-record")
    ap.add_argument("--no-tune", action="store_true", help="time the default tuning (no autotuner run)")
    ap.add_argument("--tune-iters", type=int, default=3, help="timed executions per autotuner candidate")
    ap.add_argument("--serve-duration", type=float, default=52.0,
                    help="seconds of sensor stream in the serving sub-record (>= 3,000 scans at 60 scans/s)")
    args = ap.parse_args()
    rank, world, local = dist_env()
    dist = dist_init(world)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
        barrier(dist)
        return
    if args.serve:
        if rank == 0:
            run_serve(args)
        barrier(dist)
        return
    if args.dror:
        if rank == 0:
            run_dror(args)
        barrier(dist)
        return

    import lidar_gb300 as lp

    ns = args.scans
    ctx = lp.Context(local)
    data = make_workload(ns)
    xs, rings, cfgs = [d[0] for d in data], [d[1] for d in data], [d[2] for d in data]
    pipe = lp.PipelineConfig.default()
    npts = sum(len(x) for x in xs)
    tune = None
    if not args.no_tune:
        # the library's autotuner on the workload's bucket; batches created afterwards in this
        # context (the timed batch, the end-to-end calls) take its choice
        try:
            t_tune = time.perf_counter()
            table = lp.TuningTable()
            best, rep = lp.autotune(ctx, xs, pipe, cfgs, rings, iters=args.tune_iters, table=table)
            ctx.set_tuning_table(table)
            tune = {"bucket": list(lp.tuning_key(xs, cfgs).as_tuple()), "chosen": best.as_dict(),
                    "default_ms": rep["start_ms"], "tuned_ms": rep["best_ms"], "trials": rep["trials"],
                    "iters_per_trial": args.tune_iters, "seconds": time.perf_counter() - t_tune}
        except Exception as exc:  # reported in the line; the default tuning is timed instead
            tune = {"error": leg_error(exc)}
    batch = lp.PreparedBatch(ctx, xs, pipe, cfgs, rings)
    batch_tuning = batch.tuning.as_dict()

    # per-kernel profile of one un-captured execution (dominant kernel for the roofline)
    batch.execute()
    batch.synchronize()
    prof, agg = kernel_profile(batch)
    kernels_per_step = sum(1 for n, _ in prof if n != "k_scan") + 3 * sum(1 for n, _ in prof if n == "k_scan")
    top_name = max(agg.items(), key=lambda kv: kv[1][1])[0]
    res = batch.download()
    n_obs = sum(r.n_obstacles for r in res)
    n_clusters = sum(r.n_clusters for r in res)
    n_clustered = sum(int((r.cluster_labels >= 0).sum()) for r in res)
    n_hull = sum(len(r.hull_indices) for r in res)

    batch.capture_graph()
    for _ in range(args.warmup):
        batch.execute()
    batch.synchronize()
    barrier(dist)
    with ClockSampler(local) as clocks:
        step_ms = []
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_ms.append(batch.time(1, flush_l2=False))
        wall = time.perf_counter() - t0
    barrier(dist)
    dev_ms = sum(step_ms)
    dev_ms_max = dist_max(dist, dev_ms)
    value = replica_rate(dist, world, ns * args.steps, dev_ms / 1e3)

    # the dominant kernel's launch timed with events on the context stream (roofline)
    prof2, agg2 = kernel_profile(batch)
    # a batch of 16 or more scans runs as concurrent parts: the kernel launches once per part, each
    # launch on its part's share of the work (per-launch figures are batch totals / launches)
    top_launches = agg2[top_name][0]
    top_ms = agg2[top_name][1] / top_launches
    alg = {
        "k_hull": 8 * n_clustered + 4 * n_hull + 64 * n_clusters,
        "k_jcp_rows": 20 * npts,
        "k_obs_gather": 20 * n_obs,
    }
    alg_bytes = alg.get(top_name, 20 * npts) / top_launches
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (top_ms / 1e3) / 1e9
    total_ms = sum(a[1] for a in agg2.values())
    # segmentation stage (projection + RECM + RANSAC + JCP): 20 B per input point over the summed
    # event time of its kernels in the batch (parts profiled one after the other)
    seg_ms = stage_ms(prof2, SEG_KERNELS)
    seg_gbs = 20.0 * npts / (seg_ms / 1e3) / 1e9 if seg_ms > 0 else 0.0

    plain, plain_err = [], None
    if not args.no_plain:
        # plain form: one scan per launch sequence, device-resident, no graph
        try:
            for i in range(min(ns, 32)):
                pb = lp.PreparedBatch(ctx, [xs[i]], pipe, [cfgs[i]], [rings[i]])
                pb.execute()
                pb.synchronize()
                plain.append(pb.time(3, flush_l2=False))
                pb.close()
        except Exception as exc:  # reported in the line; the batched figures stand
            plain, plain_err = [], leg_error(exc)
    plain_ms = float(np.mean(plain)) if plain else None

    e2e = None
    if not args.no_e2e:
        e2e_err, e2e_s, h2d, d2h = None, float("inf"), 0, 0
        try:
            e2e_s, h2d, d2h = e2e_leg(lp, ctx, pipe, xs, rings, cfgs, args.steps)
        except Exception as exc:  # reported in the line; the device-resident figures stand
            e2e_err = leg_error(exc)
        e2e_rate = replica_rate(dist, world, ns, e2e_s)
        if e2e_err is None and e2e_rate > 0:
            e2e = {"value": e2e_rate, "unit": "scans/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
        else:
            e2e = {"error": e2e_err or "failed on another rank", "unit": "scans/s"}

    cb = None
    if rank == 0 and not args.no_cpu:
        try:
            cb = cpu_baseline(data, budget_s=15.0)
        except Exception as exc:  # reported in the line
            cb = {"error": leg_error(exc)}

    batch.close()
    ctx.close()
    serve = dror = None
    if rank == 0 and not args.no_serve:
        try:
            serve = serve_leg(args.serve_duration)
        except Exception as exc:  # reported in the line
            serve = {"error": leg_error(exc)}
    if rank == 0 and not args.no_dror:
        try:
            dror = dror_leg(5, 3)
        except Exception as exc:  # reported in the line
            dror = {"error": leg_error(exc)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "scans/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload_name(ns), "scans": ns, "points": npts,
                       "obstacles": n_obs, "clusters": n_clusters, "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (133 MB XYZI, multi-GB working set)",
                       "graph": "captured CUDA graph per batch",
                       "tuning": batch_tuning},
            "points_per_s": world * npts * args.steps / (dev_ms_max / 1e3),
            "plain": ({"error": plain_err} if plain_err else None) if not plain else {
                "ms_per_scan": plain_ms, "scans_per_s": 1e3 / plain_ms, "p50_ms": float(np.percentile(plain, 50)),
                "p99_ms": float(np.percentile(plain, 99)), "scans": len(plain)},
            "batched_over_plain": None if not plain else (value / world) / (1e3 / plain_ms),
            "batch_latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
            "e2e": e2e,
            "gpu_launches": int(kernels_per_step * args.steps),
            "roofline": {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic_bytes(top_name, alg_bytes),
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": int(alg_bytes), "launch_ms": top_ms,
                         "stage": {"name": "segmentation (projection, RECM, RANSAC, jump convolution)",
                                   "ms": seg_ms, "algorithmic_bytes": 20 * npts, "achieved": seg_gbs,
                                   "frac": seg_gbs / peak}},
            "kernel_share": {k: round(v[1] / total_ms, 4) for k, v in sorted(agg2.items(), key=lambda kv: -kv[1][1])[:10]},
            "clocks": clocks.summary(),
            "cpu_baseline": cb,
            "autotune": tune,
            "serve": serve,
            "dror": dror,
            "wall_s": wall,
        }
        print(json.dumps(line))
    barrier(dist)


if __name__ == "__main__":
    main()
