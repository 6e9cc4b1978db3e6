"""Parity at the benchmark's full size: the whole 64-scan mixed workload that bench.py times
(8.3 M points, seeds 1000*3 + scan), run as one prepared batch (four concurrent parts) replayed from
its captured CUDA graph, equals the oracle scan by scan: segmentation and cluster labels, cluster
counts, hull index sequences and z ranges identical, calipers boxes identical, PCA box corners
within 1e-4 m. The oracle runs one scan per host thread."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


def test_full_workload_equals_oracle(ctx):
    data = [T.synth_scan(3, i) for i in range(64)]
    assert sum(len(d[0]) for d in data) > 8_000_000
    pipe = lp.PipelineConfig.default()
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b.capture_graph()
    b.execute()
    b.execute()
    got = b.download()
    b.close()
    T.oracle()
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        want = list(ex.map(lambda d: T.o_process(d[0], d[1], d[2], pipe), data))
    bad = []
    for i, (g, w) in enumerate(zip(got, want)):
        same = (np.array_equal(g.seg_labels, w.seg_labels) and np.array_equal(g.cluster_labels, w.cluster_labels)
                and g.n_clusters == w.n_clusters and np.array_equal(g.hull_offsets, w.hull_offsets)
                and np.array_equal(g.hull_indices, w.hull_indices) and np.array_equal(g.z_min, w.z_min)
                and np.array_equal(g.z_max, w.z_max)
                and all(T.boxes_identical(x, y) for x, y in zip(g.obb_calipers, w.obb_calipers))
                and all(T.box_corner_set_close(x, y, 1e-4) for x, y in zip(g.obb_pca, w.obb_pca)))
        if not same:
            bad.append(i)
    assert not bad, f"scans differing from the oracle: {bad}"
    assert sum(w.n_clusters for w in want) > 1000
