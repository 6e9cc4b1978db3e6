"""DROR at the outlier-filter configuration: 32 unorganised scans of 1.0 M points per launch (the
128-ring generator's returns shuffled, plus 5 % clutter within 15 m falling off as 1/r; synthetic
workload 4), multiplier 3 x 0.17 deg in radians, min neighbours 3, min radius 0.1 m, as one prepared
batch split into concurrent parts. Four distinct scans fill the 32 slots. Every scan's mask must
equal the reference's kd-tree search (the oracle's DROR_KDTREE mode, pinned to the reference build);
the test also reports how far that is from exact radius counting. Polar cells of these dense scans
exercise the segmentation's cell capacity."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


def test_dror_outlier_workload_equals_reference(ctx):
    uniq = [T.synth_scan(4, i) for i in range(4)]
    assert all(len(u[0]) == 1_000_000 for u in uniq)
    data = [uniq[i % 4] for i in range(32)]
    cfgs = []
    for d in data:
        c = d[2]
        c.assume_unorganized_cloud = 1
        cfgs.append(c)
    noise = lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180.0, 0.1, 3)
    pipe = lp.PipelineConfig.default(enable_noise_removal=1, noise=noise)
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, cfgs, None)
    b.execute()
    got = b.download()
    b.close()
    T.oracle()
    pts = [np.ascontiguousarray(u[0][:, :3]) for u in uniq]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        want = list(ex.map(lambda p: T.o_noise(p, noise, T.DROR_KDTREE), pts))
    for i, r in enumerate(got):
        assert np.array_equal(r.noise_labels, want[i % 4]), f"scan {i}"
    exact = T.o_noise(pts[0], noise, T.DROR_EXACT)
    print(f"scan 0: reference kd-tree marks {int(want[0].sum())} NOISE, exact counting {int(exact.sum())}, "
          f"{int((want[0] != exact).sum())} points differ")
