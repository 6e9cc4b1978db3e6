"""Serving loop (lp_server_*): scans submitted while others are on the GPU are batched together,
and every scan's results are identical to the same scan processed alone."""
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


def test_served_small_budget_splits_batches(ctx):
    """A budget that holds only one scan per slot forces single-scan batches; results unchanged."""
    data = [T.synth_scan(5, i) for i in range(20, 26)]
    pipe = lp.PipelineConfig.default()
    server = lp.Server(0, pipe, memory_budget_bytes=2 * (600 << 20), max_batch_scans=8, slots=2)
    try:
        for i, (x, ring, cfg) in enumerate(data):
            server.submit(x, ring, cfg, i)
        got = drain(server, len(data))
        stats = server.stats()
    finally:
        server.close()
    assert len(got) == len(data)
    for i, (x, ring, cfg) in enumerate(data):
        d, r = got[i]
        if d.status == lp.LP_OK:
            compare_scan(r, lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0], f"scan {i}")
        else:
            assert d.status == lp.LP_ERR_CAPACITY  # a scan larger than a slot is refused, not run
    assert stats["completed"] == len(data)
