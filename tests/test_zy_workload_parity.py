"""Parity at the benchmark's full size: the whole 64-scan mixed workload that bench.py times
(8.3 M points, seeds 1000*3 + scan), run as one prepared batch (four concurrent parts) replayed from
its captured CUDA graph, equals the oracle scan by scan: segmentation and cluster labels, cluster
counts, hull index sequences and z ranges identical, calipers boxes identical, PCA box corners
within 1e-4 m and identical to the oracle's (same binary64 steps). The oracle runs one scan per host thread. A scan that differs is run again as a
one-scan batch, and the failure message says whether its divergence repeats there."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


def first_cluster(mask):
    idx = np.nonzero(mask)[0]
    return int(idx[0]) if len(idx) else -1


def differences(g, w):
    """Which outputs of one scan differ, with counts and the first differing point or cluster."""
    d = []
    for name in ("seg_labels", "cluster_labels"):
        a, b = getattr(g, name), getattr(w, name)
        if not np.array_equal(a, b):
            ne = np.nonzero(a != b)[0]
            d.append(f"{name} {len(ne)} points from {int(ne[0])} (gpu {int(a[ne[0]])} oracle {int(b[ne[0]])})")
    if g.n_clusters != w.n_clusters:
        d.append(f"n_clusters gpu {g.n_clusters} oracle {w.n_clusters}")
        return ", ".join(d)
    k = g.n_clusters
    if not np.array_equal(g.hull_offsets, w.hull_offsets):
        c = first_cluster(g.hull_offsets != w.hull_offsets)
        d.append(f"hull_offsets from cluster {c - 1}")
    elif not np.array_equal(g.hull_indices, w.hull_indices):
        c = int(np.searchsorted(w.hull_offsets, first_cluster(g.hull_indices != w.hull_indices), side="right")) - 1
        d.append(f"hull_indices from cluster {c} (size {int(w.hull_offsets[c + 1] - w.hull_offsets[c])} vertices)")
    if not (np.array_equal(g.z_min, w.z_min) and np.array_equal(g.z_max, w.z_max)):
        d.append(f"z range from cluster {first_cluster((g.z_min != w.z_min) | (g.z_max != w.z_max))}")
    cal = [c for c in range(k) if not T.boxes_identical(g.obb_calipers[c], w.obb_calipers[c])]
    if cal:
        a, b = g.obb_calipers[cal[0]], w.obb_calipers[cal[0]]
        d.append(f"calipers boxes of {len(cal)} clusters from {cal[0]} (area gpu {a.area!r} oracle {b.area!r}, "
                 f"angle gpu {a.angle_rad!r} oracle {b.angle_rad!r})")
    pca = [c for c in range(k) if not T.box_corner_set_close(g.obb_pca[c], w.obb_pca[c], 1e-4)]
    if pca:
        d.append(f"pca boxes of {len(pca)} clusters from {pca[0]}")
    exact = [c for c in range(k) if not T.pca_boxes_equal(g.obb_pca[c], w.obb_pca[c])]
    if exact and not pca:
        d.append(f"pca boxes of {len(exact)} clusters within 1e-4 m but not identical, from {exact[0]}")
    return ", ".join(d)


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
    bad = {}
    for i, (g, w) in enumerate(zip(got, want)):
        d = differences(g, w)
        if d:
            # the scan again as a one-scan batch: a divergence of the scan itself repeats there,
            # one that depends on the batch around it does not
            x, ring, cfg = data[i]
            alone = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
            da = differences(alone, w)
            how = "exact alone" if not da else ("alone as in the batch" if not differences(alone, g) else
                                                 f"alone differently: {da}")
            bad[i] = f"{d} [{how}]"
    assert not bad, "scans differing from the oracle: " + "; ".join(f"scan {i}: {d}" for i, d in bad.items())
    assert sum(w.n_clusters for w in want) > 1000

