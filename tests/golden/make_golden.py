"""Generates the golden fixtures in this directory from the REFERENCE build (oracle/_ref/libref.so,
the reference library's own sources compiled by oracle/build_ref.sh).

Run where the reference tree exists:  python tests/golden/make_golden.py [reference data dir]

Inputs are sector crops of two reference frames (data/*.pcd) and of a synthetic scan, random
polygons, and RANSAC index-stream parameters. Every output is produced by the reference code
(segmentation, clustering, DROR, hull, antipodal pairs, calipers, PCA); ring indices are the
oracle's restatement of the ROS-only Dataloader::addRingInfo with the host libm.
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
    data = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data"
    cfg = lp.SegmenterConfig.default()
    for name, fname, lo, hi in (("kitti_000_sector", "0000000000.pcd", 0.0, 40.0),
                                ("kitti_100_sector", "0000000100.pcd", 200.0, 235.0)):
        full = T.read_pcd(os.path.join(data, fname))
        ring = T.o_ring(full, libm=T.LIBM_HOST)
        keep = sector(full, lo, hi)
        scan_case(name, np.ascontiguousarray(full[keep]), np.ascontiguousarray(ring[keep]), cfg)
    x, ring, scfg = T.synth_scan(1, 0)
    keep = sector(x, 90.0, 130.0)
    scan_case("synth_w1_sector", np.ascontiguousarray(x[keep]), np.ascontiguousarray(ring[keep]), scfg)
    polygons()
    ransac_stream()


if __name__ == "__main__":
    main()
