"""Generates the golden fixtures in this directory from the REFERENCE build (oracle/_ref/libref.so,
the reference library's own sources compiled by oracle/build_ref.sh).

Run where the reference tree exists:  python tests/golden/make_golden.py <reference data dir>
(the reference's data/ directory of .pcd frames).

Inputs are sector crops of two reference frames (data/*.pcd) and of a synthetic scan, random
polygons, two near-collinear hulls of the 64-scan workload, and RANSAC index-stream parameters.
Every output is produced by the reference code (ring indices, segmentation, clustering, DROR,
hull, antipodal pairs, calipers, PCA); ring indices come from the reference's own
Dataloader::addRingInfo, extracted from its ROS node by oracle/build_ref.sh.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import lp_testlib as T  # noqa: E402

lp = T.lp


def sector(x, lo_deg, hi_deg):
    az = np.degrees(np.arctan2(x[:, 1].astype(np.float64), x[:, 0].astype(np.float64))) % 360.0
    return (az >= lo_deg) & (az < hi_deg)


def scan_case(name, x, ring, cfg):
    out = {"xyzi": x, "ring": ring,
           "seg_cfg": np.array([getattr(cfg, f) for f, _ in lp.SegmenterConfig._fields_], np.float64)}
    lab, img = T.r_segment(x, ring, cfg, image=True)
    out["seg_labels"] = lab
    out["seg_image"] = img
    out["seg_labels_unorganized"] = T.r_segment(x, None, cfg)
    obs = np.ascontiguousarray(x[lab == lp.OBSTACLE][:, :3])
    out["cluster_labels"] = T.r_cluster(obs, lp.ClustererConfig.processor())
    pipe = lp.PipelineConfig.default()
    r = T.r_process(x, ring, cfg, pipe)
    out["pipe_seg"] = r.seg_labels
    out["pipe_cluster"] = r.cluster_labels
    out["pipe_hull_offsets"] = r.hull_offsets
    out["pipe_hull_indices"] = r.hull_indices
    out["pipe_zmin"] = r.z_min
    out["pipe_zmax"] = r.z_max
    out["pipe_calipers"] = np.array([[*b.corners_array().ravel(), b.area, b.angle_rad, b.is_valid] for b in r.obb_calipers])
    out["pipe_pca"] = np.array([[*b.corners_array().ravel(), b.area, b.angle_rad, b.is_valid] for b in r.obb_pca])
    for tag, c in (("default", lp.NoiseRemoverConfig.default()),
                   ("dense", lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180.0, 0.1, 3))):
        out["dror_" + tag] = T.r_noise(x[:, :3], c)
        shuf = np.random.default_rng(7).permutation(len(x))
        out["dror_perm"] = shuf
        out["dror_shuffled_" + tag] = T.r_noise(np.ascontiguousarray(x[shuf, :3]), c)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, len(x), "points,", r.n_clusters, "clusters")


def polygons():
    rng = np.random.default_rng(123)
    sets, hulls, pairs, cal, pca = [], [], [], [], []
    for t in range(40):
        m = int(rng.integers(3, 120))
        pts = (rng.normal(size=(m, 2)) * rng.uniform(0.2, 15.0)).astype(np.float32).astype(np.float64)
        if t % 4 == 0:
            pts = np.round(pts, 1)  # collinear runs and duplicates
        if t % 10 == 1:
            pts[:, 1] = 2.0 * pts[:, 0] + 1.0  # all collinear
        h = T.r_hull(pts)
        hp = pts[h] if len(h) else pts[:0]
        sets.append(pts)
        hulls.append(h)
        pairs.append(T.r_antipodal(hp) if len(hp) >= 2 else np.zeros((0, 2), np.int32))
        b = T.r_calipers(hp)
        cal.append([*b.corners_array().ravel(), b.area, b.angle_rad, b.is_valid])
        b = T.r_pca(hp)
        pca.append([*b.corners_array().ravel(), b.area, b.angle_rad, b.is_valid])
    np.savez_compressed(os.path.join(HERE, "polygons.npz"),
                        sizes=np.array([len(s) for s in sets]), points=np.concatenate(sets),
                        hull_sizes=np.array([len(h) for h in hulls]), hulls=np.concatenate(hulls),
                        pair_sizes=np.array([len(p) for p in pairs]), pairs=np.concatenate(pairs),
                        calipers=np.array(cal), pca=np.array(pca))
    print("polygons", len(sets))


def thin_hulls():
    """Hulls of cluster 64 of workload scan 20 and cluster 57 of scan 56 (64-scan mixed workload,
    seeds 3000 + scan): near-collinear polygons, 6-8 cm long and under a micrometre wide, with
    the reference's PCA boxes."""
    pipe = lp.PipelineConfig.default()
    hulls, boxes = [], []
    for scan, cl in ((20, 64), (56, 57)):
        x, ring, cfg = T.synth_scan(3, scan)
        r = T.r_process(x, ring, cfg, pipe)
        members = np.nonzero(r.cluster_labels == cl)[0]
        h = r.hull_indices[r.hull_offsets[cl]:r.hull_offsets[cl + 1]]
        hp = x[members, :2].astype(np.float64)[h]
        b = T.r_pca(hp)
        hulls.append(hp)
        boxes.append([*b.corners_array().ravel(), b.area, b.angle_rad, b.is_valid])
    np.savez_compressed(os.path.join(HERE, "thin_hulls.npz"), sizes=np.array([len(h) for h in hulls]),
                        points=np.concatenate(hulls), pca=np.array(boxes))
    print("thin hulls", len(hulls))


def rle(r):
    """(first positions, values) of the runs of a ring array."""
    pos = np.concatenate([[0], np.flatnonzero(np.diff(r.astype(np.int32))) + 1])
    return pos, r[pos]


def ring_streams():
    """The reference's Dataloader::addRingInfo on seeded synthetic scans (the generator is in the
    repository, so only the output is stored, run-length encoded): the single-scan and dense
    configurations, 32/64/128-ring scans of the mixed workload (the reference starts at ring 63
    whatever the sensor) and a shuffled scan (quadrant changes at random)."""
    cases = [(1, 0, False), (2, 0, False), (3, 1, False), (3, 2, False), (3, 5, False), (1, 0, True)]
    out = {"cases": np.array([[w, s, int(sh)] for w, s, sh in cases], np.int32)}
    for k, (w, sidx, sh) in enumerate(cases):
        x = T.synth_scan(w, sidx)[0]
        if sh:
            x = np.ascontiguousarray(x[np.random.default_rng(11).permutation(len(x))])
        pos, val = rle(T.r_ring(x))
        out[f"pos_{k}"], out[f"val_{k}"], out[f"n_{k}"] = pos, val, np.array(len(x))
    np.savez_compressed(os.path.join(HERE, "ring_streams.npz"), **out)
    print("ring streams", len(cases))


def ransac_stream():
    import ctypes

    o = T.oracle()
    o.lpo_ransac_draws.restype = None
    o.lpo_ransac_draws.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    ns = np.array([2, 3, 7, 100, 1000, 12345, 65537, (1 << 20) + 3, 4000000007], np.uint64)
    draws = []
    for n in ns:
        d = np.zeros(120, np.uint32)
        o.lpo_ransac_draws(int(n), 60, T.ptr(d))
        draws.append(d)
    np.savez_compressed(os.path.join(HERE, "ransac_stream.npz"), n=ns, draws=np.array(draws))
    print("ransac stream", len(ns))


def main():
    assert T.have_ref(), "oracle/_ref/libref.so missing: run oracle/build_ref.sh where the reference exists"
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference data dir>")
    data = sys.argv[1]
    cfg = lp.SegmenterConfig.default()
    for name, fname, lo, hi in (("kitti_000_sector", "0000000000.pcd", 0.0, 40.0),
                                ("kitti_100_sector", "0000000100.pcd", 200.0, 235.0)):
        full = T.read_pcd(os.path.join(data, fname))
        ring = T.r_ring(full)
        keep = sector(full, lo, hi)
        scan_case(name, np.ascontiguousarray(full[keep]), np.ascontiguousarray(ring[keep]), cfg)
    x, ring, scfg = T.synth_scan(1, 0)
    keep = sector(x, 90.0, 130.0)
    scan_case("synth_w1_sector", np.ascontiguousarray(x[keep]), np.ascontiguousarray(ring[keep]), scfg)
    polygons()
    thin_hulls()
    ring_streams()
    ransac_stream()


if __name__ == "__main__":
    main()
