"""GPU parity: every stage through the C ABI against the CPU oracle (correctly rounded libm mode)
on seeded synthetic scans and the committed reference fixtures. Integer outputs (labels,
partitions, hull index sequences, masks) must be identical; calipers boxes identical; PCA boxes
within the reference contract (corners within 1e-4 m as a set) and, beyond it, identical in
corners and area (the device follows the oracle's binary64 steps; angle within one float ulp)."""
import ctypes
import glob
import os

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


# ------------------------------------------------------------------------------- correctly rounded
def gpu_math(ctx, kind, a, b=None):
    a = np.ascontiguousarray(a, np.float32)
    bb = np.ascontiguousarray(b if b is not None else a, np.float32)
    out = np.zeros(len(a), np.float32)
    lib = lp.library()
    lib.lp_debug_math.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_void_p]
    lp.check(lib.lp_debug_math(ctx.handle, kind, T.ptr(a), T.ptr(bb), len(a), T.ptr(out)), ctx)
    return out


def oracle_math(kind, a, b=None):
    T.oracle().lpo_set_libm_mode(T.LIBM_CR)
    b = a if b is None else b
    return np.array([T.oracle().lpo_math(kind, float(x), float(y)) for x, y in zip(a, b)], np.float32)


def test_correctly_rounded_math(ctx):
    rng = np.random.default_rng(5)
    n = 20000
    y = rng.uniform(-80, 80, n).astype(np.float32)
    x = rng.uniform(-80, 80, n).astype(np.float32)
    specials = np.array([0.0, -0.0, 1e-30, -1e-30, 1.0, -1.0, 3e-8, -3e-8, 80.0], np.float32)
    y = np.concatenate([y, specials, specials * 0 + 1.0, specials])
    x = np.concatenate([x, specials * 0 + 1.0, specials, -specials])
    assert np.array_equal(gpu_math(ctx, 0, y, x).view(np.uint32), oracle_math(0, y, x).view(np.uint32))
    t = rng.uniform(-4, 4, n).astype(np.float32)
    assert np.array_equal(gpu_math(ctx, 1, t).view(np.uint32), oracle_math(1, t).view(np.uint32))
    e = -5.0 * np.sqrt(rng.uniform(0, 1, n)).astype(np.float32)
    assert np.array_equal(gpu_math(ctx, 2, e).view(np.uint32), oracle_math(2, e).view(np.uint32))
    # atan2Approx(0, 0) is 0/0: NaN payloads differ between host and device, so NaNs compare equal
    g3, o3 = gpu_math(ctx, 3, y, x), oracle_math(3, y, x)
    same = (g3.view(np.uint32) == o3.view(np.uint32)) | (np.isnan(g3) & np.isnan(o3))
    assert same.all()


def f32_bits(v):
    return int(np.array([v], np.float32).view(np.uint32)[0])


@pytest.mark.parametrize("kind,count", [(1, 1 << 32), (2, 1 << 32), (0, 1 << 31)])
def test_math_first_stage_sweep(ctx, kind, count):
    """The float-float first stage decides the rounding exactly as the binary64 / double-double
    stages do: every binary32 argument of atan and exp, 2^31 hashed atan2 pairs."""
    lib = lp.library()
    stats = (ctypes.c_uint64 * 3)()
    bad = ctypes.c_uint64()
    lp.check(lib.lp_debug_math_sweep(ctx.handle, kind, 0, count, stats, ctypes.byref(bad)), ctx)
    decided, undecided, wrong = list(stats)
    assert wrong == 0, (kind, decided, undecided, hex(bad.value))
    assert decided + undecided == count
    if kind == 2:  # the first stage covers [-87, 88.5]
        domain = (f32_bits(88.5) + 1) + (f32_bits(-87.0) - 0x80000000 + 1)
        assert undecided - (count - domain) < domain * 1e-3, (decided, undecided)
    elif kind == 1:  # and |x| in [2^-60, 2^60]
        domain = 2 * (f32_bits(2.0 ** 60) - f32_bits(2.0 ** -60) + 1)
        assert undecided - (count - domain) < domain * 1e-3, (decided, undecided)
    else:
        assert decided > count // 4, (decided, undecided)


# ------------------------------------------------------------------------------------ per stage
def scans(spec):
    return [T.synth_scan(w, s) for w, s in spec]


@pytest.mark.parametrize("w,s", [(1, 0), (3, 0), (3, 1), (3, 2)])
def test_ring_partition(ctx, w, s):
    x, _, cfg = T.synth_scan(w, s)
    first = cfg.image_height - 1
    assert np.array_equal(lp.add_ring_info(ctx, x, first), T.o_ring(x, first))


@pytest.mark.parametrize("w,s", [(1, 0), (1, 1), (2, 0), (3, 0), (3, 3), (3, 5)])
def test_segment_organized(ctx, w, s):
    x, ring, cfg = T.synth_scan(w, s)
    seg = lp.Segmenter(ctx, cfg)
    got = seg.segment(x, ring, want_image=True)
    want, img = T.o_segment(x, ring, cfg, image=True)
    assert np.array_equal(got, want)
    assert np.array_equal(seg.image(), img)


@pytest.mark.parametrize("w,s", [(1, 0), (2, 1)])
def test_segment_unorganized(ctx, w, s):
    x, _, cfg = T.synth_scan(w, s)
    got = lp.Segmenter(ctx, cfg).segment(x, None)
    assert np.array_equal(got, T.o_segment(x, None, cfg))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(T.GOLDEN, "*_sector.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_segment_reference_fixtures(ctx, path):
    """Against the reference's own outputs (the organised path uses no libm function)."""
    g = dict(np.load(path))
    cfg = lp.SegmenterConfig(*[float(v) if t is not ctypes.c_int32 else int(v)
                               for v, (_, t) in zip(g["seg_cfg"], lp.SegmenterConfig._fields_)])
    seg = lp.Segmenter(ctx, cfg)
    assert np.array_equal(seg.segment(g["xyzi"], g["ring"], want_image=True), g["seg_labels"])
    assert np.array_equal(seg.image(), g["seg_image"])


@pytest.mark.parametrize("w,s", [(1, 0), (2, 0), (3, 4)])
def test_cluster(ctx, w, s):
    x, ring, cfg = T.synth_scan(w, s)
    lab = T.o_segment(x, ring, cfg)
    obs = np.ascontiguousarray(x[lab == lp.OBSTACLE][:, :3])
    c = lp.ClustererConfig.processor()
    got = lp.Clusterer(ctx, c).cluster(obs)
    want = T.o_cluster(obs, c)
    assert np.array_equal(got, want)


def test_cluster_voxel_capacity(ctx):
    """More than 200,000 occupied voxels: the reference throws std::overflow_error
    (static_unordered_map.hpp:81); the library reports LP_ERR_CAPACITY (OverflowError)."""
    rng = np.random.default_rng(0)
    pts = rng.uniform(-80, 80, size=(260000, 3)).astype(np.float32)
    with pytest.raises(OverflowError):
        lp.Clusterer(ctx, lp.ClustererConfig(0.05, 0.25, 0.25, 3)).cluster(pts)
    with pytest.raises(OverflowError):
        T.o_cluster(pts, lp.ClustererConfig(0.05, 0.25, 0.25, 3))


def kdtree_clouds():
    """Clouds for the tree build: tiny sizes around the build's thresholds (3, 64, 2048 points),
    coordinates with many ties (the tree then depends on nth_element's swaps), a dense scan."""
    rng = np.random.default_rng(17)
    out = []
    for n in (1, 2, 3, 4, 5, 64, 65, 66, 2047, 2048, 2049, 4097, 5000, 70000):
        out.append((f"uniform{n}", rng.uniform(-50, 50, size=(n, 3)).astype(np.float32)))
    for n in (300, 9000, 150000):
        out.append((f"ties{n}", np.round(rng.normal(size=(n, 3)) * 4.0, 0).astype(np.float32)))
    x = T.synth_scan(1, 0)[0]
    out.append(("scan", np.ascontiguousarray(x[:, :3])))
    return out


@pytest.mark.parametrize("name,pts", kdtree_clouds(), ids=lambda v: v if isinstance(v, str) else "")
def test_kdtree_build_matches_reference(ctx, name, pts):
    """The device kd-tree equals the reference's KDTree::rebuild (std::nth_element per node) node
    for node, including where coordinates tie; subtree sizes follow the range arithmetic."""
    nodes, sizes = lp.debug_kdtree(ctx, pts)
    want = T.o_kdtree_positions(pts)
    assert np.array_equal(nodes.view(np.uint32), want.view(np.uint32)), name
    n = len(pts)
    expect = np.zeros(n, np.uint32)
    todo = [(0, n)]
    while todo:
        b, e = todo.pop()
        if e <= b:
            continue
        m = b + (e - b) // 2
        expect[m] = e - b
        todo += [(b, m), (m + 1, e)]
    assert np.array_equal(sizes, expect), name


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(T.GOLDEN, "*_sector.npz"))), ids=os.path.basename)
def test_noise_removal_reference_fixtures(ctx, path):
    """DROR masks equal the reference's own NoiseRemover output (made by the reference build) on
    the fixtures' clouds, in input order and shuffled, default and dense configurations."""
    g = np.load(path)
    x = np.ascontiguousarray(g["xyzi"][:, :3])
    perm = g["dror_perm"]
    for tag, c in (("default", lp.NoiseRemoverConfig.default()),
                   ("dense", lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180.0, 0.1, 3))):
        nr = lp.NoiseRemover(ctx, c)
        assert np.array_equal(nr.filter(x), g["dror_" + tag]), tag
        assert np.array_equal(nr.filter(np.ascontiguousarray(x[perm])), g["dror_shuffled_" + tag]), tag


def test_noise_removal_organized_scan(ctx):
    """A whole organised scan in ring order (long runs of neighbouring queries: deep leftover
    stacks): the mask equals the reference kd-tree's, which here differs from exact counting."""
    x = np.ascontiguousarray(T.synth_scan(1, 0)[0][:, :3])
    c = lp.NoiseRemoverConfig.default()
    got = lp.NoiseRemover(ctx, c).filter(x)
    assert np.array_equal(got, T.o_noise(x, c, T.DROR_KDTREE))


@pytest.mark.parametrize("cfg", [lp.NoiseRemoverConfig.default(), lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180, 0.1, 3)],
                         ids=["default", "dense"])
def test_noise_removal_exact(ctx, cfg):
    x, _, _ = T.synth_scan(1, 0)
    rng = np.random.default_rng(3)
    clutter = rng.normal(size=(3000, 3)) * 6.0
    pts = np.ascontiguousarray(np.concatenate([x[:, :3], clutter]).astype(np.float32))
    pts = np.ascontiguousarray(pts[rng.permutation(len(pts))])
    got = lp.NoiseRemover(ctx, cfg).filter(pts)
    assert np.array_equal(got, T.o_noise(pts, cfg, T.DROR_KDTREE))
    assert got.sum() > 0


@pytest.mark.parametrize("k", [2, 5, 9])
def test_noise_removal_grid_ties(ctx, k):
    """Points on a half-metre grid with duplicates, shuffled, and a fixed radius of 1 m: many
    neighbours lie at exactly the radius (counted, as d <= r2) and subtree boxes touch the radius
    exactly, the test the walks use to skip subtrees; larger min_neighbours leave more points short
    and more candidates for the ordered chain (stops followed by candidates that run out)."""
    rng = np.random.default_rng(40 + k)
    g = rng.integers(-24, 25, size=(30000, 3)).astype(np.float32) * 0.5
    g[:, 2] *= 0.25
    dup = g[rng.integers(0, len(g), size=6000)]
    sparse = rng.uniform(-40, 40, size=(4000, 3)).astype(np.float32)
    pts = np.concatenate([g, dup, sparse])
    pts = np.ascontiguousarray(pts[rng.permutation(len(pts))])
    cfg = lp.NoiseRemoverConfig(1e-6, 1.0, k)
    got = lp.NoiseRemover(ctx, cfg).filter(pts)
    want = T.o_noise(pts, cfg, T.DROR_KDTREE)
    assert np.array_equal(got, want)
    assert 0 < got.sum() < len(pts)


def test_polygons(ctx):
    rng = np.random.default_rng(11)
    poly = lp.Polygonizer(ctx)
    for t in range(30):
        m = int(rng.integers(3, 400))
        pts = (rng.normal(size=(m, 2)) * rng.uniform(0.2, 15.0)).astype(np.float32).astype(np.float64)
        if t % 3 == 0:
            pts = np.round(pts, 1)
        h = poly.convexHull(pts)
        assert np.array_equal(h, T.o_hull(pts))
        hp = np.ascontiguousarray(pts[h])
        if len(hp) >= 2:
            assert np.array_equal(poly.findAntipodalPairsOfConvexHull(hp), T.o_antipodal(hp))
        assert T.boxes_identical(poly.boundingBoxRotatingCalipers(hp), T.o_calipers(hp))
        pb = poly.boundingBoxPrincipalComponentAnalysis(hp)
        assert T.box_corner_set_close(pb, T.o_pca(hp)[0], 1e-4)
        assert T.pca_boxes_equal(pb, T.o_pca(hp)[0])


def test_hull_ties_follow_reference_sort(ctx):
    """Clouds full of identical points (coordinates rounded to a coarse grid): which of the identical
    points the hull reports follows the reference's std::sort order (libstdc++ introsort replayed on
    the device), index for index, up to 40,000 points (ranges partitioned by the whole CTA)."""
    rng = np.random.default_rng(29)
    poly = lp.Polygonizer(ctx)
    differ = 0
    for t, n in enumerate([5, 17, 40, 300, 2047, 2049, 5000, 40000]):
        pts = np.round(rng.normal(size=(n, 2)) * 3.0, 0 if t % 2 else 1).astype(np.float32).astype(np.float64)
        got = poly.convexHull(pts)
        want = T.o_hull(pts, T.TIES_LIBSTDCXX)
        assert np.array_equal(got, want), n
        differ += int(not np.array_equal(want, T.o_hull(pts, T.TIES_INDEX)))
    assert differ > 0  # the input-order rule would differ on some of these
    # degenerate clouds: every point identical (the hull is [first, last] of one coordinate), two
    # distinct points repeated, a vertical line of repeated points
    for n in [3, 4, 17, 50, 3000]:
        one = np.repeat(np.array([[1.25, -0.5]]), n, 0)
        two = np.array([[0.5, 0.5], [2.0, -1.0]])[rng.integers(0, 2, n)]
        two[:2] = [[0.5, 0.5], [2.0, -1.0]]
        line = np.stack([np.full(n, 3.0), np.round(rng.normal(size=n) * 2.0)], 1)
        for pts in (one, two, line):
            assert np.array_equal(poly.convexHull(pts), T.o_hull(pts, T.TIES_LIBSTDCXX)), n


def test_pipeline_hull_ties(ctx):
    """A scan with copies of half its obstacle points at the same (x, y), 0.5 m higher and one ring
    up (so each copy wins its own range-image pixel and joins the cluster): clusters hold many
    identical (x, y), and the hulls follow the reference's std::sort order among them (more than
    a hundred hull indices differ under an input-order rule)."""
    x, ring, cfg = T.synth_scan(3, 3)
    pipe = lp.PipelineConfig.default()
    base = T.o_process(x, ring, cfg, pipe)
    obs = np.nonzero(base.seg_labels == lp.OBSTACLE)[0]
    dup = np.sort(np.random.default_rng(4).choice(obs, size=len(obs) // 2, replace=False))
    cp = x[dup].copy()
    cp[:, 2] += 0.5
    rc = np.maximum(ring[dup].astype(np.int32) - 1, 0).astype(np.uint16)
    x2 = np.ascontiguousarray(np.concatenate([x, cp]))
    r2 = np.ascontiguousarray(np.concatenate([ring, rc]))
    got = lp.process_batch(ctx, [x2], pipe, [cfg], [r2])[0]
    want = T.o_process(x2, r2, cfg, pipe, ties=T.TIES_LIBSTDCXX)
    compare_scan(got, want, "copies above the obstacles")
    other = T.o_process(x2, r2, cfg, pipe, ties=T.TIES_INDEX)
    assert int((want.hull_indices != other.hull_indices).sum()) > 50


def test_pca_thin_hulls(ctx):
    """The two near-collinear hulls of the 64-scan workload (tests/golden/thin_hulls.npz, 6-8 cm
    long and under a micrometre wide) through lp_bounding_box_pca: the reference's box."""
    g = np.load(os.path.join(T.GOLDEN, "thin_hulls.npz"))
    off = np.concatenate([[0], np.cumsum(g["sizes"])])
    poly = lp.Polygonizer(ctx)
    for t in range(len(g["sizes"])):
        hp = np.ascontiguousarray(g["points"][off[t]:off[t + 1]])
        pb = poly.boundingBoxPrincipalComponentAnalysis(hp)
        assert T.pca_boxes_equal(pb, T.o_pca(hp)[0]), t
        assert np.array_equal(pb.corners_array(), g["pca"][t][:8].reshape(4, 2)), t


def test_pca_workload_scans_exact(ctx):
    """Scans 20 and 56 of the 64-scan workload, whose thin clusters 64 and 57 once gave PCA boxes
    beyond 1e-4 m: every PCA box of both scans (warp path of the hull kernel) equals the oracle's."""
    pipe = lp.PipelineConfig.default()
    for s in (20, 56):
        x, ring, cfg = T.synth_scan(3, s)
        got = lp.process_batch(ctx, [x], pipe, [cfg], [ring])[0]
        want = T.o_process(x, ring, cfg, pipe)
        assert got.n_clusters == want.n_clusters
        bad = [c for c in range(want.n_clusters) if not T.pca_boxes_equal(got.obb_pca[c], want.obb_pca[c])]
        assert not bad, (s, bad[:5])


@pytest.mark.parametrize("w,s", [(1, 0), (3, 0)])
def test_split_clouds(ctx, w, s):
    """Ground / obstacle / unsegmented clouds (processor.cpp:558-579) from a segmentation: each label
    class's points in input order with its colour; empty input; a NULL output buffer only counts."""
    x, ring, cfg = T.synth_scan(w, s)
    lab = lp.Segmenter(ctx, cfg).segment(x, ring)
    got = lp.split_clouds(ctx, x, lab)
    classes = [(lab == lp.GROUND, (124, 252, 0)), (lab == lp.OBSTACLE, (200, 0, 0)),
               ((lab != lp.GROUND) & (lab != lp.OBSTACLE), (255, 255, 0))]
    assert sum(len(c) for c in got) == len(x)
    for cloud, (sel, rgb) in zip(got, classes):
        want = x[sel]
        assert len(cloud) == len(want)
        for k, f in enumerate("xyz"):
            assert np.array_equal(cloud[f], want[:, k])
        assert (cloud["r"] == rgb[0]).all() and (cloud["g"] == rgb[1]).all() and (cloud["b"] == rgb[2]).all()
        assert (cloud["a"] == 255).all()
    empty = lp.split_clouds(ctx, x[:0], lab[:0])
    assert all(len(c) == 0 for c in empty)
    counts = np.zeros(3, np.uint32)
    a = np.ascontiguousarray(x, np.float32)
    lp.check(lp.library().lp_split_clouds(ctx.handle, T.ptr(a), T.ptr(lab), len(a), None, None, None, T.ptr(counts)), ctx)
    assert counts.tolist() == [int(c[0].sum()) for c in classes]


@pytest.mark.parametrize("layout", ["xyzir_aligned", "xyzr_unaligned"])
def test_unpack_pointcloud2(ctx, layout):
    """PointCloud2 bytes (padded rows, fields at their offsets, aligned or not) unpacked as
    convert<PointT> does (processor.cpp:42-179); a field outside the record is rejected."""
    x, ring, _ = T.synth_scan(1, 0)
    width, height = 1000, len(x) // 1000
    n = width * height
    if layout == "xyzir_aligned":
        point_step, offs = 32, dict(x=0, y=4, z=8, intensity=16, ring=20)
    else:
        point_step, offs = 15, dict(x=1, y=5, z=9, intensity=lp.NO_FIELD, ring=13)
    row_step = width * point_step + 7
    buf = np.zeros(height * row_step, np.uint8)
    for r in range(height):
        rec = buf[r * row_step:r * row_step + width * point_step].reshape(width, point_step)
        pts = x[r * width:(r + 1) * width]
        for k, f in enumerate("xyz"):
            rec[:, offs[f]:offs[f] + 4] = pts[:, k].astype("<f4").view(np.uint8).reshape(width, 4)
        if offs["intensity"] != lp.NO_FIELD:
            rec[:, offs["intensity"]:offs["intensity"] + 4] = pts[:, 3].astype("<f4").view(np.uint8).reshape(width, 4)
        rec[:, offs["ring"]:offs["ring"] + 2] = ring[r * width:(r + 1) * width].astype("<u2").view(np.uint8).reshape(width, 2)
    xyzi, rg = lp.unpack_pointcloud2(ctx, buf, width, height, point_step, row_step, **offs)
    want = x[:n].copy()
    if offs["intensity"] == lp.NO_FIELD:
        want[:, 3] = 0.0
    assert np.array_equal(xyzi.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(rg, ring[:n])
    with pytest.raises(ValueError):  # LP_ERR_BAD_ARG
        lp.unpack_pointcloud2(ctx, buf, width, height, point_step, row_step, x=point_step - 2)


# ------------------------------------------------------------------------------------- pipeline
def compare_scan(got, want, label=""):
    assert np.array_equal(got.seg_labels, want.seg_labels), label
    assert np.array_equal(got.cluster_labels, want.cluster_labels), label
    assert got.n_clusters == want.n_clusters, label
    assert np.array_equal(got.hull_offsets, want.hull_offsets), label
    assert np.array_equal(got.hull_indices, want.hull_indices), label
    assert np.array_equal(got.z_min, want.z_min) and np.array_equal(got.z_max, want.z_max), label
    for a, b in zip(got.obb_calipers, want.obb_calipers):
        assert T.boxes_identical(a, b), label
    for a, b in zip(got.obb_pca, want.obb_pca):
        assert T.box_corner_set_close(a, b, 1e-4), label
        assert T.pca_boxes_equal(a, b), label


def test_pipeline_batch_mixed(ctx):
    spec = [(3, i) for i in range(8)]
    data = scans(spec)
    pipe = lp.PipelineConfig.default()
    res = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    for (x, ring, cfg), r, sp in zip(data, res, spec):
        compare_scan(r, T.o_process(x, ring, cfg, pipe), str(sp))


def test_pipeline_computed_rings(ctx):
    data = scans([(1, 2), (3, 6)])
    pipe = lp.PipelineConfig.default(compute_ring=1)
    res = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], None)
    for (x, _, cfg), r in zip(data, res):
        rings = T.o_ring(x, cfg.image_height - 1)
        compare_scan(r, T.o_process(x, rings, cfg, lp.PipelineConfig.default()))


def test_pipeline_with_noise_removal(ctx):
    data = scans([(1, 3), (3, 7)])
    pipe = lp.PipelineConfig.default(enable_noise_removal=1,
                                     noise=lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180, 0.1, 3))
    res = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    for (x, ring, cfg), r in zip(data, res):
        want = T.o_process(x, ring, cfg, pipe, dror_mode=T.DROR_KDTREE)
        assert np.array_equal(r.noise_labels, want.noise_labels)
        compare_scan(r, want)


def test_batch_equals_alone(ctx):
    data = scans([(3, 8), (3, 9), (3, 10)])
    pipe = lp.PipelineConfig.default()
    batched = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    for d, b in zip(data, batched):
        alone = lp.process_batch(ctx, [d[0]], pipe, [d[2]], [d[1]])[0]
        compare_scan(b, alone)


def test_pinned_reused_outputs(ctx):
    """Page-locked inputs and result buffers reused across calls give the fresh-buffer results."""
    data = scans([(3, 4), (3, 5)])
    pipe = lp.PipelineConfig.default()
    want = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    px = [lp.pinned_copy(d[0]) for d in data]
    pr = [lp.pinned_copy(d[1]) for d in data]
    bufs = [lp.ResultBuffers(len(d[0]), pinned=True) for d in data]
    for _ in range(2):  # the second call overwrites the first call's results in place
        lp.process_batch(ctx, px, pipe, [d[2] for d in data], pr, outputs=bufs, raw=True)
        for b, w in zip(bufs, want):
            compare_scan(b.result(), w)


def test_pinned_split_batch(ctx):
    """16 or more scans on page-locked buffers run as concurrent parts (scans dealt round-robin,
    each part reading and writing the caller's buffers on its own stream): the results, call after
    call into the same buffers, are those of the unsplit pageable path in the caller's order."""
    data = scans([(1, i) for i in range(6)] + [(3, i) for i in range(10, 24)])
    pipe = lp.PipelineConfig.default()
    want = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    px = [lp.pinned_copy(d[0]) for d in data]
    pr = [lp.pinned_copy(d[1]) for d in data]
    bufs = [lp.ResultBuffers(len(d[0]), pinned=True) for d in data]
    for _ in range(2):
        lp.process_batch(ctx, px, pipe, [d[2] for d in data], pr, outputs=bufs, raw=True)
        for i, (b, w) in enumerate(zip(bufs, want)):
            compare_scan(b.result(), w, f"scan {i}")


def test_batch_composition_independent(ctx):
    """A scan's results do not depend on which scans share its batch or on what earlier batches
    left in device memory (sizes 18k-201k points, several groupings, after a large unrelated
    batch has been run through the same buffers)."""
    data = [T.synth_scan(5, i) for i in range(10, 17)]
    pipe = lp.PipelineConfig.default()
    alone = [lp.process_batch(ctx, [d[0]], pipe, [d[2]], [d[1]])[0] for d in data]
    junk = [T.synth_scan(3, i) for i in range(4)]
    for grp in ([1, 2], [2, 3], [0, 1, 2], [1, 2, 3, 4], [0, 1, 2, 3, 4, 5, 6]):
        lp.process_batch(ctx, [d[0] for d in junk], pipe, [d[2] for d in junk], [d[1] for d in junk])
        res = lp.process_batch(ctx, [data[i][0] for i in grp], pipe, [data[i][2] for i in grp],
                               [data[i][1] for i in grp])
        for i, r in zip(grp, res):
            compare_scan(r, alone[i], f"scan {10 + i} in group {grp}")


@pytest.mark.parametrize("step", [1.0 / 16.0, 0.05])
def test_pipeline_quantized(ctx, step):
    """Coordinates on a grid: on the 1/16 m grid every coordinate difference is exact and many hull
    candidates are exactly collinear; on the 5 cm grid they are near-collinear. Both drive the
    hull chain's orientation test into its near-tie branches."""
    pipe = lp.PipelineConfig.default()
    for s in (0, 1):
        x, ring, cfg = T.synth_scan(3, s)
        q = x.copy()
        q[:, :3] = (np.round(x[:, :3].astype(np.float64) / step) * step).astype(np.float32)
        got = lp.process_batch(ctx, [q], pipe, [cfg], [ring])[0]
        compare_scan(got, T.o_process(q, ring, cfg, pipe), f"scan {s} step {step}")


def test_edge_cases(ctx):
    x, ring, cfg = T.synth_scan(1, 0)
    pipe = lp.PipelineConfig.default()
    far = x[np.hypot(x[:, 0], x[:, 1]) > 30.0]
    cases = [
        (x[:0], ring[:0]),                     # empty scan
        (x[:1], ring[:1]),                     # one point
        (x[:2], ring[:2]),                     # two points
        (far, ring[np.hypot(x[:, 0], x[:, 1]) > 30.0]),  # no near-field RANSAC candidates
        (x[x[:, 2] < -1.5], ring[x[:, 2] < -1.5]),        # ground only
    ]
    xs = [np.ascontiguousarray(c[0]) for c in cases]
    rs = [np.ascontiguousarray(c[1]) for c in cases]
    res = lp.process_batch(ctx, xs, pipe, [cfg] * len(xs), rs)
    for xx, rr, r in zip(xs, rs, res):
        compare_scan(r, T.o_process(xx, rr, cfg, pipe), f"n={len(xx)}")


def test_cpp_dropin_example(ctx, tmp_path):
    """The C++ drop-in classes (cpp/lidar_processing_gpu.hpp) reproduce the pipeline's labels and
    hull indices: the example's checksum equals one computed from lp_process_batch."""
    import subprocess

    x, ring, cfg = T.synth_scan(1, 5)
    (tmp_path / "x.bin").write_bytes(x.tobytes())
    (tmp_path / "r.bin").write_bytes(ring.tobytes())
    exe = os.path.join(T.PKG, "example_processor")
    out = subprocess.run([exe, str(tmp_path / "x.bin"), str(tmp_path / "r.bin"), str(cfg.image_height),
                          str(cfg.image_width)], capture_output=True, text=True, check=True).stdout
    r = lp.process_batch(ctx, [x], lp.PipelineConfig.default(compute_obb=0), [cfg], [ring])[0]
    h = 1469598103934665603
    mask = (1 << 64) - 1

    def mix(v):
        nonlocal h
        h = ((h ^ (int(v) & 0xFFFFFFFF)) * 1099511628211) & mask

    for v in r.seg_labels:
        mix(v)
    for v in r.cluster_labels[r.seg_labels == lp.OBSTACLE]:
        mix(v)
    for k in range(r.n_clusters):
        for v in r.hull(k):
            mix(v)
    assert f"clusters {r.n_clusters} " in out
    assert out.strip().endswith(f"checksum {h:016x}"), out


def test_prepared_batch_split(ctx):
    """A batch of 16 or more scans runs as concurrent parts on their own streams (scans dealt
    round-robin): its results, with and without a captured graph, equal lp_process_batch's in the
    caller's scan order."""
    data = scans([(1, i) for i in range(6)] + [(3, i) for i in range(14)])
    pipe = lp.PipelineConfig.default()
    ref = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    assert b.points == sum(len(d[0]) for d in data)
    b.execute()
    got = b.download()
    b.capture_graph()
    b.execute()
    b.execute()
    got2 = b.download()
    for i, (r, g1, g2) in enumerate(zip(ref, got, got2)):
        compare_scan(g1, r, f"scan {i}")
        compare_scan(g2, r, f"scan {i} (graph)")
    prof = b.profile()
    assert sum(1 for n, _ in prof if n == "k_hull") == 2  # 20 scans: two parts
    b.close()


def test_prepared_batch_split_noise(ctx):
    """A split prepared batch with the outlier filter enabled (each part filters its own scans before
    segmenting them) equals the unsplit batch, and its first scans equal the oracle."""
    data = scans([(1, i) for i in range(16)])
    pipe = lp.PipelineConfig.default(enable_noise_removal=1,
                                     noise=lp.NoiseRemoverConfig(3 * 0.17 * np.pi / 180, 0.1, 3))
    ref = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b.capture_graph()
    b.execute()
    got = b.download()
    for i, (r, g) in enumerate(zip(ref, got)):
        assert np.array_equal(g.noise_labels, r.noise_labels), i
        compare_scan(g, r, f"scan {i}")
    for (x, ring, cfg), g in list(zip(data, got))[:2]:
        want = T.o_process(x, ring, cfg, pipe, dror_mode=T.DROR_KDTREE)
        assert np.array_equal(g.noise_labels, want.noise_labels)
        compare_scan(g, want)
    b.close()


def test_prepared_batch_and_graph(ctx):
    """lp_batch_create / execute / capture_graph give the same results as lp_process_batch."""
    data = scans([(3, 11), (1, 4)])
    pipe = lp.PipelineConfig.default()
    ref = lp.process_batch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b = lp.PreparedBatch(ctx, [d[0] for d in data], pipe, [d[2] for d in data], [d[1] for d in data])
    b.execute()
    got = b.download()
    b.capture_graph()
    b.execute()
    b.execute()
    got2 = b.download()
    for r, g1, g2 in zip(ref, got, got2):
        compare_scan(g1, r)
        compare_scan(g2, r)
    b.close()
