"""Pins the CPU oracle (oracle/lp_oracle.cpp) against fixtures produced by the reference library's
own code (tests/golden/make_golden.py over oracle/_ref). The oracle runs with the host libm, as
the reference does; all comparisons are exact except the PCA box (Eigen's JacobiSVD is restated),
whose corners are compared as a set within 1e-9 m."""
import glob
import os

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
CASES = sorted(glob.glob(os.path.join(T.GOLDEN, "*_sector.npz")))


def load(path):
    return dict(np.load(path))


def seg_cfg(g):
    return lp.SegmenterConfig(*[float(v) if t is not lp.ctypes.c_int32 else int(v)
                                for v, (_, t) in zip(g["seg_cfg"], lp.SegmenterConfig._fields_)])


def box_from(row):
    b = lp.BoundingBox()
    for k in range(4):
        b.corners[k][0], b.corners[k][1] = row[2 * k], row[2 * k + 1]
    b.area, b.angle_rad, b.is_valid = row[8], row[9], int(row[10])
    return b


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p))
def test_segmentation_pinned(built, path):
    g = load(path)
    cfg = seg_cfg(g)
    lab, img = T.o_segment(g["xyzi"], g["ring"], cfg, libm=T.LIBM_HOST, image=True)
    assert np.array_equal(lab, g["seg_labels"])
    assert np.array_equal(img, g["seg_image"])
    assert np.array_equal(T.o_segment(g["xyzi"], None, cfg, libm=T.LIBM_HOST), g["seg_labels_unorganized"])


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p))
def test_clustering_pinned(built, path):
    g = load(path)
    obs = np.ascontiguousarray(g["xyzi"][g["seg_labels"] == lp.OBSTACLE][:, :3])
    assert np.array_equal(T.o_cluster(obs, lp.ClustererConfig.processor(), libm=T.LIBM_HOST), g["cluster_labels"])


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p))
def test_pipeline_pinned(built, path):
    g = load(path)
    r = T.o_process(g["xyzi"], g["ring"], seg_cfg(g), lp.PipelineConfig.default(), libm=T.LIBM_HOST)
    assert np.array_equal(r.seg_labels, g["pipe_seg"])
    assert np.array_equal(r.cluster_labels, g["pipe_cluster"])
    assert np.array_equal(r.hull_offsets, g["pipe_hull_offsets"])
    assert np.array_equal(r.hull_indices, g["pipe_hull_indices"])
    assert np.array_equal(r.z_min, g["pipe_zmin"]) and np.array_equal(r.z_max, g["pipe_zmax"])
    for b, row in zip(r.obb_calipers, g["pipe_calipers"]):
        assert T.boxes_identical(b, box_from(row))
    for b, row in zip(r.obb_pca, g["pipe_pca"]):
        assert T.box_corner_set_close(b, box_from(row), 1e-9)


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p))
def test_dror_kdtree_pinned(built, path):
    """The reference kd-tree search keeps its traversal stack across queries (kdtree.hpp:339-397);
    the oracle's kd-tree mode reproduces that exactly, in input order and shuffled."""
    g = load(path)
    x = np.ascontiguousarray(g["xyzi"][:, :3])
    perm = g["dror_perm"]
    for tag, c in (("default", lp.NoiseRemoverConfig.default()),
                   ("dense", lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180.0, 0.1, 3))):
        assert np.array_equal(T.o_noise(x, c, T.DROR_KDTREE), g["dror_" + tag])
        assert np.array_equal(T.o_noise(np.ascontiguousarray(x[perm]), c, T.DROR_KDTREE), g["dror_shuffled_" + tag])


def test_polygons_pinned(built):
    g = load(os.path.join(T.GOLDEN, "polygons.npz"))
    off = np.concatenate([[0], np.cumsum(g["sizes"])])
    hoff = np.concatenate([[0], np.cumsum(g["hull_sizes"])])
    poff = np.concatenate([[0], np.cumsum(g["pair_sizes"])])
    for t in range(len(g["sizes"])):
        pts = g["points"][off[t]:off[t + 1]]
        h = T.o_hull(pts)
        want = g["hulls"][hoff[t]:hoff[t + 1]]
        # identical hull point sequences; indices identical where no duplicate points exist
        assert np.array_equal(pts[h], pts[want])
        if len(np.unique(pts, axis=0)) == len(pts):
            assert np.array_equal(h, want)
        hp = pts[want]
        if len(hp) >= 2:
            assert np.array_equal(T.o_antipodal(hp), g["pairs"][poff[t]:poff[t + 1]])
        assert T.boxes_identical(T.o_calipers(hp), box_from(g["calipers"][t]))
        assert T.box_corner_set_close(T.o_pca(hp)[0], box_from(g["pca"][t]), 1e-9)


# ------------------------------------------------------------------ RANSAC index stream restatement
class Mt19937:
    """MT19937 (Matsumoto & Nishimura 1998), as restated in the device kernel."""

    def __init__(self, seed):
        self.mt = [0] * 624
        self.mt[0] = seed
        for i in range(1, 624):
            self.mt[i] = (1812433253 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self.idx = 624

    def next(self):
        if self.idx >= 624:
            for i in range(624):
                y = (self.mt[i] & 0x80000000) | (self.mt[(i + 1) % 624] & 0x7FFFFFFF)
                self.mt[i] = self.mt[(i + 397) % 624] ^ (y >> 1) ^ (0x9908B0DF if y & 1 else 0)
            self.idx = 0
        y = self.mt[self.idx]
        self.idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF

    def bounded(self, rng):
        """Lemire's nearly divisionless draw in [0, rng)."""
        m = self.next() * rng
        low = m & 0xFFFFFFFF
        if low < rng:
            t = ((1 << 32) - rng) % rng
            while low < t:
                m = self.next() * rng
                low = m & 0xFFFFFFFF
        return m >> 32


def test_ransac_index_stream_matches_libstdcxx():
    """The device RANSAC draws (MT19937 + Lemire bounded draw) equal std::mt19937{42} with
    std::uniform_int_distribution<uint32_t>{0, n-1} (segmenter.cpp:369-386) as recorded from the
    reference toolchain."""
    g = load(os.path.join(T.GOLDEN, "ransac_stream.npz"))
    for n, want in zip(g["n"], g["draws"]):
        n = int(n)
        if n > 0xFFFFFFFF:
            continue
        gen = Mt19937(42)
        got = []
        for _ in range(60):
            a = gen.bounded(n)
            b = gen.bounded(n)
            while b == a:
                b = gen.bounded(n)
            got += [a, b]
        assert got == want.tolist(), n


# --------------------------------------------------------------------------- PCA covariance error
def test_pca_covariance_error(built):
    """The PCA box's 2x2 covariance as the FP64 oracle forms it (mean, then centred sums in vertex
    order, divided by n - 1; the device forms the same sums in the same order) against exact
    rational arithmetic, on the 40 golden polygons' hulls and on car-sized footprints with float32
    coordinates 5-80 m from the sensor. Error relative to the larger diagonal entry: 2.8e-16 at
    most on these inputs (one rounding), checked below 1e-14."""
    from fractions import Fraction

    g = load(os.path.join(T.GOLDEN, "polygons.npz"))
    off = np.concatenate([[0], np.cumsum(g["sizes"])])
    hoff = np.concatenate([[0], np.cumsum(g["hull_sizes"])])
    polys = []
    for t in range(len(g["sizes"])):
        pts = g["points"][off[t]:off[t + 1]]
        polys.append(pts[g["hulls"][hoff[t]:hoff[t + 1]]])
    rng = np.random.default_rng(11)
    for _ in range(40):
        r, az, yaw = rng.uniform(5, 80), rng.uniform(0, 2 * np.pi), rng.uniform(0, np.pi)
        u = rng.uniform(-2.25, 2.25, 60)
        v = rng.uniform(-0.9, 0.9, 60)
        x = r * np.cos(az) + u * np.cos(yaw) - v * np.sin(yaw)
        y = r * np.sin(az) + u * np.sin(yaw) + v * np.cos(yaw)
        xy = np.stack([x, y], 1).astype(np.float32).astype(np.float64)
        polys.append(xy[T.o_hull(xy)])
    worst = 0.0
    for hp in polys:
        n = len(hp)
        if n < 3:
            continue
        _, cov = T.o_pca(hp)
        xs = [Fraction(float(v)) for v in hp[:, 0]]
        ys = [Fraction(float(v)) for v in hp[:, 1]]
        mx, my = sum(xs) / n, sum(ys) / n
        exact = [sum((a - mx) ** 2 for a in xs) / (n - 1), sum((a - mx) * (b - my) for a, b in zip(xs, ys)) / (n - 1),
                 sum((b - my) ** 2 for b in ys) / (n - 1)]
        scale = max(abs(exact[0]), abs(exact[2]))
        worst = max(worst, max(float(abs(Fraction(float(c)) - e) / scale) for c, e in zip(cov, exact)))
    assert worst < 1e-14, worst


# ------------------------------------------------------- whole workload against the reference's code
def test_workload_matches_reference_code(built):
    """The oracle (host-libm mode) against the reference's own classes built from its sources
    (oracle/_ref) on all 64 scans of the benchmark workload: segmentation and cluster labels,
    cluster counts, z ranges and hull offsets identical; hull index sequences identical except
    where a cluster holds two points with the same (x, y) (the reference's std::sort leaves their
    order to the library; the hull's point sequence is identical there too); calipers boxes
    identical and PCA corners within 1e-9 m, both being functions of the hull's points. With the
    oracle's libstdc++ tie order the hull index sequences are identical everywhere."""
    if not os.path.exists(T.REF_PATH):
        pytest.skip("reference build absent (oracle/build_ref.sh needs the reference tree)")
    from concurrent.futures import ThreadPoolExecutor

    pipe = T.lp.PipelineConfig.default()
    data = [T.synth_scan(3, i) for i in range(64)]
    T.oracle()
    T.ref()
    # the reference build runs on one thread (it crashes when several threads run their own
    # instances); the oracle is thread-safe
    ref = [T.r_process(d[0], d[1], d[2], pipe) for d in data]
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        orc = list(ex.map(lambda d: T.o_process(d[0], d[1], d[2], pipe, libm=T.LIBM_HOST), data))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        orc_lib = list(ex.map(lambda d: T.o_process(d[0], d[1], d[2], pipe, libm=T.LIBM_HOST,
                                                    ties=T.TIES_LIBSTDCXX), data))
    T.oracle().lpo_set_hull_ties(T.TIES_INDEX)
    for i, (a, c) in enumerate(zip(ref, orc_lib)):
        assert np.array_equal(a.hull_indices, c.hull_indices), i
    ties = 0
    for i, ((x, _, _), a, b) in enumerate(zip(data, ref, orc)):
        for k in ("seg_labels", "cluster_labels", "hull_offsets", "z_min", "z_max"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), (i, k)
        assert a.n_clusters == b.n_clusters, i
        obs = x[a.seg_labels == T.lp.OBSTACLE]
        for c in range(a.n_clusters):
            lo, hi = a.hull_offsets[c], a.hull_offsets[c + 1]
            ha, hb = a.hull_indices[lo:hi], b.hull_indices[lo:hi]
            if not np.array_equal(ha, hb):
                pts = obs[a.cluster_labels[a.seg_labels == T.lp.OBSTACLE] == c][:, :2]
                assert len(np.unique(pts, axis=0)) < len(pts), (i, c)
                assert np.array_equal(pts[ha], pts[hb]), (i, c)
                ties += 1
            assert T.boxes_identical(a.obb_calipers[c], b.obb_calipers[c]), (i, c)
            assert T.box_corner_set_close(a.obb_pca[c], b.obb_pca[c], 1e-9), (i, c)
    assert ties <= 1, ties  # one cluster of 5,120 with the libstdc++ 13 build here


# ------------------------------------------------- std::sort restatement (order of equivalent points)
def tie_heavy_inputs():
    rng = np.random.default_rng(21)
    sizes = [0, 1, 2, 3, 15, 16, 17, 18, 31, 32, 33, 63, 64, 65, 100, 257, 1000, 3000]
    for n in sizes:
        for distinct in (1, 2, 3, 7, 50, 10_000):
            xy = rng.integers(0, distinct, size=(n, 2)).astype(np.float64) * 0.25
            yield xy
            yield xy[np.lexsort((xy[:, 1], xy[:, 0]))]          # sorted
            yield xy[np.lexsort((xy[:, 1], xy[:, 0]))][::-1]    # reverse sorted
    for n in (40, 200, 2000):  # organ pipe and saw-tooth in x with duplicated y
        x = np.concatenate([np.arange(n // 2), np.arange(n // 2)[::-1]]).astype(np.float64)
        yield np.stack([x, np.zeros_like(x)], 1)
        x = (np.arange(n) % 7).astype(np.float64)
        yield np.stack([x, (np.arange(n) % 3).astype(np.float64)], 1)


def test_introsort_restatement_matches_std_sort(built):
    """The restated libstdc++ introsort (oracle/introsort.h) leaves the reference comparator's
    equivalent elements exactly where std::sort does, and its heapsort path matches libstdc++'s."""
    count = 0
    for xy in tie_heavy_inputs():
        assert np.array_equal(T.o_debug_sort(xy, 0), T.o_debug_sort(xy, 1)), len(xy)
        if len(xy) > 16:  # shorter ranges never reach the introsort loop, so never its heapsort
            assert np.array_equal(T.o_debug_sort(xy, 2), T.o_debug_sort(xy, 3)), len(xy)
        count += 1
    assert count > 300


def test_hull_tie_mode_matches_reference_hull(built):
    """With libstdc++ tie order the oracle's hull equals the reference's convexHull index for
    index, duplicates included."""
    if not os.path.exists(T.REF_PATH):
        pytest.skip("reference build absent (oracle/build_ref.sh needs the reference tree)")
    rng = np.random.default_rng(8)
    for t in range(200):
        n = int(rng.integers(3, 400))
        xy = rng.integers(0, int(rng.integers(2, 30)), size=(n, 2)).astype(np.float64) * 0.5
        assert np.array_equal(T.o_hull(xy, ties=T.TIES_LIBSTDCXX), T.r_hull(xy)), t


def ring_runs(r):
    pos = np.concatenate([[0], np.flatnonzero(np.diff(r.astype(np.int32))) + 1])
    return pos, r[pos]


def test_ring_pinned_to_reference_dataloader(built):
    """The oracle's ring partition (start ring 63, host libm) equals the reference's own
    Dataloader::addRingInfo output on the committed seeded scans, including 32- and 128-ring
    sensors (where the reference still counts down from 63) and a shuffled scan."""
    g = np.load(os.path.join(T.GOLDEN, "ring_streams.npz"))
    for k, (w, s, shuffled) in enumerate(g["cases"]):
        x = T.synth_scan(int(w), int(s))[0]
        if shuffled:
            x = np.ascontiguousarray(x[np.random.default_rng(11).permutation(len(x))])
        assert len(x) == int(g[f"n_{k}"])
        pos, val = ring_runs(T.o_ring(x, first_ring=63, libm=T.LIBM_HOST))
        assert np.array_equal(pos, g[f"pos_{k}"]) and np.array_equal(val, g[f"val_{k}"]), (w, s, shuffled)


def test_ring_oracle_matches_reference_code_on_sector_fixtures(built):
    """Where the reference build is present, the extracted Dataloader::addRingInfo and the oracle
    agree on the fixtures' point sequences (crops, so the rings restart at 63)."""
    if not T.have_ref():
        pytest.skip("reference build not present")
    for path in CASES:
        x = load(path)["xyzi"]
        assert np.array_equal(T.r_ring(x), T.o_ring(x, first_ring=63, libm=T.LIBM_HOST)), path


def test_thin_hulls_pca_pinned(built):
    """Two near-collinear hulls of the 64-scan workload (6-8 cm long, under a micrometre wide):
    the oracle's PCA box equals the reference's (JacobiSVD restated from Eigen 3.4)."""
    g = np.load(os.path.join(T.GOLDEN, "thin_hulls.npz"))
    off = np.concatenate([[0], np.cumsum(g["sizes"])])
    for t in range(len(g["sizes"])):
        hp = g["points"][off[t]:off[t + 1]]
        b, _ = T.o_pca(hp)
        want = box_from(g["pca"][t])
        assert np.array_equal(b.corners_array(), want.corners_array()) and b.area == want.area, t


def svd_check(a, v):
    """V orthonormal, columns eigenvectors of the symmetric a, eigenvalues descending."""
    assert np.allclose(v.T @ v, np.eye(2), atol=1e-15)
    lam = np.array([v[:, 0] @ a @ v[:, 0], v[:, 1] @ a @ v[:, 1]])
    scale = np.abs(a).max()
    assert np.allclose(a @ v, v * lam, atol=4e-16 * scale)
    assert lam[0] >= lam[1] - 4e-16 * scale


def test_jacobi_svd2_restatement(built):
    """Eigen's JacobiSVD of a 2x2 covariance as the oracle restates it: a diagonal input keeps its
    axes (columns swapped when the second value is larger), an off-diagonal entry at or below
    2 eps max|diagonal| (after scaling) is not rotated, however close to isotropic the matrix is,
    one just above it is rotated; equal singular values keep their columns; a non-finite input is
    invalid; random symmetric matrices give orthonormal eigenvectors with descending values."""
    eps = np.finfo(np.float64).eps
    assert np.array_equal(T.o_svd2([[3.0, 0.0], [0.0, 1.0]]), np.eye(2))
    assert np.array_equal(T.o_svd2([[1.0, 0.0], [0.0, 3.0]]), [[0.0, 1.0], [1.0, 0.0]])
    assert np.array_equal(T.o_svd2([[2.0, 0.0], [0.0, 2.0]]), np.eye(2))
    assert np.array_equal(T.o_svd2([[0.0, 0.0], [0.0, 0.0]]), np.eye(2))
    # near-isotropic, off-diagonal at the threshold: no rotation (a closed-form angle gives 45 deg)
    assert np.array_equal(T.o_svd2([[1.0, 2 * eps], [2 * eps, 1.0]]), np.eye(2))
    assert np.array_equal(T.o_svd2([[1.0, 1e-20], [1e-20, 1.0 - 1e-15]]), np.eye(2))
    # just above it: a 45-degree rotation
    v = T.o_svd2([[1.0, 4 * eps], [4 * eps, 1.0]])
    assert np.allclose(np.abs(v), np.sqrt(0.5), atol=1e-12)
    assert T.o_svd2([[np.nan, 0.0], [0.0, 1.0]]) is None
    assert T.o_svd2([[np.inf, 0.0], [0.0, 1.0]]) is None
    rng = np.random.default_rng(5)
    for _ in range(2000):
        sxx, syy = rng.uniform(0, 10, 2) ** rng.uniform(-3, 3, 2)
        sxy = rng.normal() * np.sqrt(sxx * syy) * rng.uniform(0, 1) ** 4
        a = np.array([[sxx, sxy], [sxy, syy]])
        svd_check(a, T.o_svd2(a))


def test_glibc_rand_restatement_matches_libc():
    """The oracle's restatement of glibc's rand() (the stream the processor's cluster colours draw
    from, processor.cpp:630-632, never seeded) equals the host C library's rand() after srand(1)."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srand(1)
    seq = np.array([libc.rand() for _ in range(5000)], np.int32)
    assert np.array_equal(T.o_glibc_rand(0, 5000), seq)
    assert np.array_equal(T.o_glibc_rand(4321, 100), seq[4321:4421])
