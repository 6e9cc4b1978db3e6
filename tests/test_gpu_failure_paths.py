"""Bounded device waits give up and report instead of hanging: the look-back prefix scan whose
predecessor tile never publishes, and an mbarrier wait without an arrival, each polled a few times.
The call returns LP_ERR_TIMEOUT and the context stays usable (a scan processed right after equals the
oracle). No GPU fault or hang is provoked: the waits are bounded and touch only their own state."""
import ctypes

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


def _wait_timeout(ctx, kind, limit):
    f = lp.library().lp_debug_wait_timeout
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_uint32, ctypes.c_void_p]
    gave_up = ctypes.c_uint32(0)
    st = f(ctx.handle, kind, limit, ctypes.byref(gave_up))
    return st, gave_up.value


@pytest.mark.parametrize("kind", [0, 1], ids=["lookback-scan", "mbarrier"])
def test_bounded_wait_runs_out_and_reports(ctx, kind):
    st, gave_up = _wait_timeout(ctx, kind, 64)
    assert st == lp.LP_ERR_TIMEOUT and gave_up != 0
    # the context is still usable and exact afterwards
    x, ring, cfg = T.synth_scan(1, 0)
    keep = (x[:, 0] > 0) & (x[:, 1] > 0)
    x, ring = np.ascontiguousarray(x[keep]), np.ascontiguousarray(ring[keep])
    pipe = lp.PipelineConfig.default()
    got = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
    want = T.o_process(x, ring, cfg, pipe)
    assert np.array_equal(got.seg_labels, want.seg_labels)
    assert np.array_equal(got.cluster_labels, want.cluster_labels)
    assert np.array_equal(got.hull_indices, want.hull_indices)


def test_bounded_wait_arguments(ctx):
    assert _wait_timeout(ctx, 2, 64)[0] == lp.LP_ERR_BAD_ARG
    assert _wait_timeout(ctx, 0, 0)[0] == lp.LP_ERR_BAD_ARG
