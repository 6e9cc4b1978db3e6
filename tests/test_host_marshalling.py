"""Host-side argument marshalling of lp_process_batch (Python mirror), checked on CPU against a
stand-in for the shared library that records what it is handed: the per-scan lp_scan_input and
lp_scan_output structs point at the caller's arrays, a bound BatchCall hands over the same structs
on every run, counts the library writes reach the result buffers, and inputs a bound call could
only read through a stale conversion copy are refused."""
import ctypes

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp


class RecordingLibrary:
    def __init__(self):
        self.calls = []

    def lp_process_batch(self, handle, pipeline_ref, ins, outs, n):
        self.calls.append((ctypes.addressof(pipeline_ref._obj), ctypes.addressof(ins), ctypes.addressof(outs), n,
                           [(ins[i].xyzi, ins[i].ring, ins[i].n, bytes(ins[i].seg)) for i in range(n)],
                           [bytes(outs[i]) for i in range(n)]))
        for i in range(n):  # what the library reports back per scan
            outs[i].n_obstacles = 10 + i
            outs[i].n_clusters = i
            outs[i].n_hull_indices = 3 * i
            outs[i].status = 0
        return 0


class FakeContext:
    handle = None


@pytest.fixture
def rec(monkeypatch):
    r = RecordingLibrary()
    monkeypatch.setattr(lp, "library", lambda: r)
    return r


def scans():
    rng = np.random.default_rng(3)
    xs = [rng.normal(size=(n, 4)).astype(np.float32) for n in (5, 0, 17)]
    rs = [np.arange(len(x), dtype=np.uint16) for x in xs]
    cfgs = [lp.SegmenterConfig.default() for _ in xs]
    cfgs[2].image_width = 1024
    return xs, rs, cfgs


def addr(a):
    return a.__array_interface__["data"][0]


def test_batch_call_structs_point_at_the_callers_arrays(rec):
    xs, rs, cfgs = scans()
    bufs = [lp.ResultBuffers(len(x)) for x in xs]
    want_out = [bytes(b.out) for b in bufs]
    call = lp.BatchCall(xs, None, cfgs, [rs[0], None, rs[2]], outputs=bufs)
    got = call.run(FakeContext())
    assert got is call.bufs
    _, _, _, n, ins, outs = rec.calls[0]
    assert n == 3
    assert [i[0] for i in ins] == [addr(x) for x in xs]
    assert [i[1] for i in ins] == [addr(rs[0]), None, addr(rs[2])]
    assert [i[2] for i in ins] == [5, 0, 17]
    assert [i[3] for i in ins] == [bytes(c) for c in cfgs]
    assert outs == want_out
    assert [(b.out.n_obstacles, b.out.n_clusters, b.out.n_hull_indices) for b in bufs] == [(10, 0, 0), (11, 1, 3),
                                                                                          (12, 2, 6)]


def test_batch_call_reruns_with_the_same_structs(rec):
    xs, rs, cfgs = scans()
    bufs = [lp.ResultBuffers(len(x), pinned=False) for x in xs]
    call = lp.BatchCall(xs, lp.PipelineConfig.default(), cfgs, rs, outputs=bufs)
    call.run(FakeContext())
    call.run(FakeContext())
    a, b = rec.calls
    assert a[:4] == b[:4] and a[4] == b[4]
    # the second call hands over the first call's structs with the counts the library wrote into them
    for i, (before, after) in enumerate(zip(a[5], b[5])):
        o = lp.ScanOutput.from_buffer_copy(before)
        o.n_obstacles, o.n_clusters, o.n_hull_indices, o.status = 10 + i, i, 3 * i, 0
        assert after == bytes(o)


def test_process_batch_converts_and_matches_batch_call(rec):
    xs, rs, cfgs = scans()
    bufs = [lp.ResultBuffers(len(x)) for x in xs]
    res = lp.process_batch(FakeContext(), xs, None, cfgs, rs, outputs=bufs, raw=True)
    assert res == bufs
    lp.BatchCall(xs, None, cfgs, rs, outputs=[lp.ResultBuffers(len(x)) for x in xs]).run(FakeContext())
    p, q = rec.calls
    assert p[3] == q[3] and p[4] == q[4]
    # inputs that need converting go through process_batch, which converts them first
    x3 = [x[:, :3].astype(np.float64) for x in xs]
    lp.process_batch(FakeContext(), x3, None, cfgs, [r.astype(np.int64) for r in rs], raw=True)
    _, _, _, n, ins, _ = rec.calls[2]
    assert n == 3 and [i[2] for i in ins] == [5, 0, 17]


@pytest.mark.parametrize("bad", ["n3", "f64", "strided", "ring_i32"])
def test_batch_call_refuses_inputs_it_would_copy(rec, bad):
    xs, rs, cfgs = scans()
    if bad == "n3":
        xs[0] = np.ascontiguousarray(xs[0][:, :3])
    elif bad == "f64":
        xs[0] = xs[0].astype(np.float64)
    elif bad == "strided":
        xs[0] = np.zeros((5, 8), np.float32)[:, ::2]
    else:
        rs[0] = rs[0].astype(np.int32)
    with pytest.raises(ValueError):
        lp.BatchCall(xs, None, cfgs, rs)
    assert not rec.calls


class PinningLibrary(RecordingLibrary):
    """Also hands out 'page-locked' blocks (plain host memory here) as lp_host_alloc would."""

    def __init__(self):
        super().__init__()
        self.blocks = []

    def lp_host_alloc(self, nbytes, out):
        b = ctypes.create_string_buffer(int(nbytes) + 256)
        self.blocks.append(b)
        ctypes.cast(out, ctypes.POINTER(ctypes.c_void_p))[0] = (ctypes.addressof(b) + 255) // 256 * 256
        return 0

    def lp_host_free(self, p):
        pass


def test_bench_end_to_end_leg(monkeypatch):
    """bench.py's end-to-end leg: page-locked copies of the scans and rings, one bound call run
    once untimed plus max(3, steps // 2) timed steps, and the bytes it reports per step."""
    import os
    import sys

    sys.path.insert(0, T.REPO)
    import bench

    lib = PinningLibrary()
    monkeypatch.setattr(lp, "library", lambda: lib)
    xs, rs, cfgs = scans()
    secs, h2d, d2h = bench.e2e_leg(lp, FakeContext(), lp.PipelineConfig.default(), xs, rs, cfgs, steps=8)
    assert len(lib.calls) == 1 + 4 and secs >= 0.0
    ins = lib.calls[0][4]
    assert [i[2] for i in ins] == [5, 0, 17]
    assert all(i[0] != addr(x) for i, x in zip(ins, xs))  # the page-locked copies, not the originals
    assert h2d == sum(x.nbytes + r.nbytes for x, r in zip(xs, rs))
    # counts the stand-in reports: clusters 0, 1, 2 and hull indices 0, 3, 6
    want = sum(9 * len(x) + 4 * (k + 1 + 3 * k) + 8 * k + 144 * k for k, x in enumerate(xs))
    assert d2h == want
    assert os.path.basename(bench.__file__) == "bench.py"
