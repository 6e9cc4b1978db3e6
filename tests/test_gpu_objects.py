"""The processor's per-cluster products (processor.cpp:609-797) through lp_cluster_objects against the
oracle's restatement of that loop: the clustered cloud (points grouped by label in input order, colours
from glibc's rand() stream at a given draw offset), the vehicle gates (calipers over each candidate
cluster's raw points, the vehicle table) and the boundary marker points, on scans of the 64-scan
workload where the gates box several clusters; offsets that move forward and back in the rand() stream."""
import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu

SCANS = [22, 3, 11, 9]


def compare(got, want):
    assert np.array_equal(got.cloud, want.cloud)
    assert np.array_equal(got.vehicle_class, want.vehicle_class)
    for c, (a, b) in enumerate(zip(got.gate_boxes, want.gate_boxes)):
        assert T.boxes_identical(a, b), c
    assert np.array_equal(got.marker_offsets, want.marker_offsets)
    assert np.array_equal(got.marker_points, want.marker_points)


@pytest.mark.parametrize("gates", [True, False], ids=["gates", "no-gates"])
def test_cluster_objects_match_oracle(ctx, gates):
    pipe = lp.PipelineConfig.default()
    boxed = 0
    for k, s in enumerate(SCANS):
        x, ring, cfg = T.synth_scan(3, s)
        r = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
        draws = [0, 3 * 1000 + 7, 17][k % 3]  # ahead, then behind the context's cached position
        got = lp.cluster_objects(ctx, x, r, vehicle_gates=gates, rand_draws=draws)
        want = T.o_cluster_objects(x, r, vehicle_gates=gates, rand_draws=draws)
        compare(got, want)
        assert len(got.cloud) == int((r.cluster_labels >= 0).sum())
        boxed += int((got.vehicle_class >= 0).sum())
        if not gates:
            assert (got.vehicle_class == -1).all()
    if gates:
        assert boxed >= 10  # the gate path ran to a classification on these scans


def test_cluster_objects_colours_continue_the_rand_stream(ctx):
    """Consecutive frames: the second scan's colours start where the first scan's 3K draws ended."""
    pipe = lp.PipelineConfig.default()
    x, ring, cfg = T.synth_scan(3, 22)
    r = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
    first = lp.cluster_objects(ctx, x, r, rand_draws=0)
    second = lp.cluster_objects(ctx, x, r, rand_draws=3 * int(r.n_clusters))
    draws = T.o_glibc_rand(0, 6 * int(r.n_clusters)) % 256
    lab_first = np.searchsorted(np.cumsum(np.bincount(r.cluster_labels[r.cluster_labels >= 0])), np.arange(len(first.cloud)), side="right")
    for objs, base in ((first, 0), (second, 3 * int(r.n_clusters))):
        rgb = np.stack([objs.cloud["r"], objs.cloud["g"], objs.cloud["b"]], 1).astype(np.int64)
        want = draws[base:base + 3 * int(r.n_clusters)].reshape(-1, 3)[lab_first]
        assert np.array_equal(rgb, want)


def test_cluster_objects_empty_and_capacity(ctx):
    x, ring, cfg = T.synth_scan(3, 3)
    r = lp.process_batch(ctx, [x], lp.PipelineConfig.default(), [cfg], [ring])[0]
    # a marker buffer too small is reported with the size it needs
    import ctypes
    a = np.ascontiguousarray(x, np.float32)
    K = int(r.n_clusters)
    out, bufs = lp.object_buffers(len(a), K, r.hull_offsets)
    out.marker_capacity = 5
    lab = np.ascontiguousarray(r.cluster_labels, np.int32)
    hoff = np.ascontiguousarray(r.hull_offsets[: K + 1], np.uint32)
    hidx = np.ascontiguousarray(r.hull_indices, np.int32)
    zmin = np.ascontiguousarray(r.z_min[:K], np.float32)
    zmax = np.ascontiguousarray(r.z_max[:K], np.float32)
    st = lp.library().lp_cluster_objects(ctx.handle, T.ptr(a), T.ptr(lab), len(a), K, T.ptr(hoff), T.ptr(hidx),
                                         T.ptr(zmin), T.ptr(zmax), ctypes.byref(lp.ObjectConfig(0, 0, 0)),
                                         ctypes.byref(out))
    assert st == lp.LP_ERR_CAPACITY and out.n_marker_points > 5
    # a label at or beyond n_clusters is rejected
    bad = lab.copy()
    bad[np.nonzero(bad >= 0)[0][0]] = K
    out2, _ = lp.object_buffers(len(a), K, r.hull_offsets)
    st = lp.library().lp_cluster_objects(ctx.handle, T.ptr(a), T.ptr(bad), len(a), K, T.ptr(hoff), T.ptr(hidx),
                                         T.ptr(zmin), T.ptr(zmax), ctypes.byref(lp.ObjectConfig(0, 0, 0)),
                                         ctypes.byref(out2))
    assert st == lp.LP_ERR_BAD_ARG
