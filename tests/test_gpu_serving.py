"""Serving loop (lp_server_*): scans submitted while others are on the GPU are batched together,
every scan's results equal the oracle's and the same scan processed alone, and admission is by the
memory free in the server's pool: a scan that does not fit the memory free now waits and then
completes exactly; only a scan larger than the whole budget is refused."""
import time

import numpy as np
import pytest

import lp_testlib as T
from test_gpu_parity import compare_scan

lp = T.lp
pytestmark = pytest.mark.gpu


def drain(server, want, timeout_s=60.0):
    got = {}
    t0 = time.time()
    while len(got) < want and time.time() - t0 < timeout_s:
        for d, r in server.poll(wait_us=2000):
            got[int(d.tag)] = (d, r)
    return got


def test_served_results_equal_alone(ctx):
    data = [T.synth_scan(5, i) for i in range(20)]
    pipe = lp.PipelineConfig.default()
    server = lp.Server(0, pipe, memory_budget_bytes=6 << 30, max_batch_scans=8, slots=2)
    try:
        for i, (x, ring, cfg) in enumerate(data):  # burst: most arrive while earlier batches run
            server.submit(x, ring, cfg, i)
        got = drain(server, len(data))
        stats = server.stats()
    finally:
        server.close()
    assert len(got) == len(data)
    assert stats["completed"] == len(data) and stats["failed"] == 0
    assert stats["max_batch_seen"] > 1, stats  # continuous batching actually batched
    for i, (x, ring, cfg) in enumerate(data):
        d, r = got[i]
        assert d.status == lp.LP_OK and d.latency_ms > 0
        alone = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
        compare_scan(r, alone, f"scan {i} (batch of {d.batch_scans})")
        compare_scan(r, T.o_process(x, ring, cfg, pipe), f"scan {i} against the oracle")


def scan_bytes(ctx, x, ring, cfg, pipe):
    return batch_bytes(ctx, [(x, ring, cfg)], pipe)


def batch_bytes(ctx, data, pipe):
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    try:
        return b.device_bytes
    finally:
        b.close()


def test_large_scan_waits_for_memory_then_completes(ctx):
    """A pool that holds the largest scan, and a batch of four small scans, but not both: the large
    scan, queued right behind the small ones (the server held while the burst is submitted), waits
    for their memory instead of being refused, then completes; every result equals the oracle."""
    pipe = lp.PipelineConfig.default()
    small = [T.synth_scan(5, i) for i in range(30, 34)]
    sizes = [(len(d[0]), k) for k, d in enumerate(T.synth_scan(5, i) for i in range(34, 48))]
    big = T.synth_scan(5, 34 + max(sizes)[1])
    need_big = scan_bytes(ctx, *big, pipe)
    need_small = batch_bytes(ctx, small, pipe)
    budget = max(need_big, need_small) + min(need_big, need_small) // 2  # either alone fits, not both
    server = lp.Server(0, pipe, memory_budget_bytes=budget, max_batch_scans=4, slots=2)
    try:
        data = small + [big]
        server.hold()  # the burst queues as a whole: the small batch starts first, the big scan is next
        for i, (x, ring, cfg) in enumerate(data):
            server.submit(x, ring, cfg, i)
        server.hold(False)
        got = drain(server, len(data))
        stats = server.stats()
    finally:
        server.close()
    assert len(got) == len(data) and stats["failed"] == 0, stats
    assert stats["batches"] >= 2, stats
    d_big, r_big = got[len(data) - 1]
    assert d_big.status == lp.LP_OK
    # it did not fit beside the batch ahead of it: the queue's head waited for that batch's memory
    assert stats["memory_waits"] >= 1, stats
    for i, (x, ring, cfg) in enumerate(data):
        d, r = got[i]
        assert d.status == lp.LP_OK
        compare_scan(r, T.o_process(x, ring, cfg, pipe), f"scan {i}")


def test_scan_larger_than_budget_is_refused(ctx):
    """Only a scan that exceeds the whole budget is refused; the scans around it still run."""
    pipe = lp.PipelineConfig.default()
    data = [T.synth_scan(5, i) for i in range(20, 24)]
    need = max(scan_bytes(ctx, *d, pipe) for d in data)
    big = T.synth_scan(5, 46)  # 322,827 points
    server = lp.Server(0, pipe, memory_budget_bytes=need + (need >> 3), max_batch_scans=8, slots=2)
    try:
        order = data[:2] + [big] + data[2:]
        for i, (x, ring, cfg) in enumerate(order):
            server.submit(x, ring, cfg, i)
        got = drain(server, len(order))
        stats = server.stats()
    finally:
        server.close()
    assert len(got) == len(order) and stats["completed"] == len(order)
    too_big = scan_bytes(ctx, *big, pipe) > need + (need >> 3)
    assert too_big
    for i, (x, ring, cfg) in enumerate(order):
        d, r = got[i]
        if i == 2 and too_big:
            assert d.status == lp.LP_ERR_CAPACITY
        else:
            assert d.status == lp.LP_OK
            compare_scan(r, T.o_process(x, ring, cfg, pipe), f"scan {i}")
