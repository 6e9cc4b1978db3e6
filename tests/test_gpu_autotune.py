"""Run-time tuning on the GPU: every tuning gives the default tuning's results (the oracle's), a
context's tuning table reaches the batches created afterwards (prepared batches and the page-locked
split path), and lp_autotune returns a valid tuning no slower than where it started, stored under
the scans' bucket."""
import numpy as np
import pytest

import lp_testlib as T
from test_gpu_parity import compare_scan, scans

lp = T.lp
pytestmark = pytest.mark.gpu

TUNINGS = [
    dict(parts=2, balance_parts=1),
    dict(parts=3),
    dict(parts=5, balance_parts=1, hull_cta_min=64),
    dict(hull_cta_min=128, hull_ctas_per_sm=1),
    dict(cell_ctas_per_sm=1, jcp_ctas_per_sm=16, hull_ctas_per_sm=4),
    dict(parts=1, hull_cta_min=256, cell_ctas_per_sm=12, jcp_ctas_per_sm=3),
]


def run(ctx, data, pipe, tuning=None, graph=False):
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data], tuning=tuning)
    try:
        t = b.tuning
        if graph:
            b.capture_graph()
        b.execute()
        return t, b.download()
    finally:
        b.close()


def test_tunings_give_identical_results(ctx):
    data = [T.synth_scan(5, i) for i in range(60, 80)]  # 20 mixed scans
    pipe = lp.PipelineConfig.default()
    t0, want = run(ctx, data, pipe)
    assert t0.as_dict() == lp.Tuning.default().as_dict()
    for i in (0, 7, 13):
        compare_scan(want[i], T.o_process(data[i][0], data[i][1], data[i][2], pipe), f"scan {i} against the oracle")
    for kw in TUNINGS:
        t = lp.Tuning.default(**kw)
        got_t, got = run(ctx, data, pipe, tuning=t, graph=True)
        assert got_t.as_dict() == t.as_dict()
        for i in range(len(data)):
            compare_scan(got[i], want[i], f"{kw} scan {i}")


def test_context_table_applies(ctx):
    data = scans([(1, i) for i in range(6)] + [(3, i) for i in range(10, 24)])
    pipe = lp.PipelineConfig.default()
    xs, rings, cfgs = [d[0] for d in data], [d[1] for d in data], [d[2] for d in data]
    want = lp.process_batch(ctx, xs, pipe, cfgs, rings)
    key = lp.tuning_key(xs, cfgs)
    tuned = lp.Tuning.default(parts=3, balance_parts=1, hull_cta_min=128)
    tab = lp.TuningTable()
    tab.set(key, tuned, 1.0)
    ctx.set_tuning_table(tab)
    try:
        t, got = run(ctx, data, pipe)
        assert t.as_dict() == tuned.as_dict()
        for i, (g, w) in enumerate(zip(got, want)):
            compare_scan(g, w, f"prepared scan {i}")
        # the page-locked path splits into the table's parts too, results in the caller's order
        px = [lp.pinned_copy(x) for x in xs]
        pr = [lp.pinned_copy(r) for r in rings]
        bufs = [lp.ResultBuffers(len(x), pinned=True) for x in xs]
        lp.process_batch(ctx, px, pipe, cfgs, pr, outputs=bufs, raw=True)
        for i, (b, w) in enumerate(zip(bufs, want)):
            compare_scan(b.result(), w, f"page-locked scan {i}")
        # a batch of another bucket keeps the defaults
        t1, _ = run(ctx, data[:1], pipe)
        assert t1.as_dict() == lp.Tuning.default().as_dict()
    finally:
        ctx.set_tuning_table(None)
    t2, _ = run(ctx, data, pipe)
    assert t2.as_dict() == lp.Tuning.default().as_dict()


def test_autotune(ctx):
    data = [T.synth_scan(5, i) for i in range(80, 96)]  # 16 scans: the part split is a candidate
    pipe = lp.PipelineConfig.default()
    xs, rings, cfgs = [d[0] for d in data], [d[1] for d in data], [d[2] for d in data]
    tab = lp.TuningTable()
    best, rep = lp.autotune(ctx, xs, pipe, cfgs, rings, iters=2, table=tab)
    assert best.valid()
    assert rep["trials"] >= 10 and len(rep["candidates"]) == rep["trials"]
    assert rep["candidates"][0][0] == lp.Tuning.default().as_dict()
    assert all(ms > 0 for _, ms in rep["candidates"])
    assert rep["best_ms"] <= rep["start_ms"]
    # the choice is one of the timed candidates, stored under the scans' bucket
    assert best.as_dict() in [c for c, _ in rep["candidates"]]
    found, t, ms = tab.get(lp.tuning_key(xs, cfgs))
    assert found and t.as_dict() == best.as_dict() and ms == pytest.approx(rep["best_ms"])
    # installed, it reaches the next batch, with the default tuning's results
    _, want = run(ctx, data, pipe)
    ctx.set_tuning_table(tab)
    try:
        t_used, got = run(ctx, data, pipe, graph=True)
    finally:
        ctx.set_tuning_table(None)
    assert t_used.as_dict() == best.as_dict()
    for i, (g, w) in enumerate(zip(got, want)):
        compare_scan(g, w, f"tuned scan {i}")
