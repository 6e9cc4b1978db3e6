"""Test helpers: bindings of the CPU oracle (oracle/liblp_oracle.so), of the reference build
(oracle/_ref/libref.so, present only where the reference tree was available at build time), the
package's synthetic scan generator, a PCD reader and comparison helpers."""
from __future__ import annotations

import ctypes
import itertools
import os
import sys

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "lidar-processing-v2_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)

import lidar_gb300 as lp  # noqa: E402
from lidar_gb300 import ptr  # noqa: E402

ORACLE_PATH = os.path.join(REPO, "oracle", "liblp_oracle.so")
REF_PATH = os.path.join(REPO, "oracle", "_ref", "libref.so")
GOLDEN = os.path.join(REPO, "tests", "golden")

LIBM_CR, LIBM_HOST = 0, 1
TIES_INDEX, TIES_LIBSTDCXX = 0, 1  # order of hull points with equal (x, y): input order / the reference's std::sort
DROR_EXACT, DROR_KDTREE = 0, 1  # exact radius counting / the reference's kd-tree search (its stack kept)

_oracle = None
_ref = None


def oracle():
    global _oracle
    if _oracle is None:
        o = ctypes.CDLL(ORACLE_PATH)
        P, c = ctypes.c_void_p, ctypes
        sig = {
            "lpo_set_libm_mode": (None, [c.c_int]),
            "lpo_set_hull_ties": (None, [c.c_int]),
            "lpo_debug_sort": (c.c_int32, [P, c.c_uint32, c.c_int, P]),
            "lpo_cr_ambiguous_count": (c.c_long, []),
            "lpo_math": (c.c_float, [c.c_int, c.c_float, c.c_float]),
            "lpo_add_ring_info": (c.c_int32, [P, c.c_uint32, c.c_uint16, P]),
            "lpo_segment": (c.c_int32, [P, P, c.c_uint32, P, P, P]),
            "lpo_noise_remove": (c.c_int32, [P, c.c_uint32, c.c_uint32, P, c.c_int, P]),
            "lpo_cluster": (c.c_int32, [P, c.c_uint32, c.c_uint32, P, P]),
            "lpo_convex_hull": (c.c_int32, [P, c.c_uint32, P, P]),
            "lpo_antipodal_pairs": (c.c_int32, [P, c.c_uint32, P, c.c_uint32, P]),
            "lpo_bounding_box_rotating_calipers": (c.c_int32, [P, c.c_uint32, P]),
            "lpo_bounding_box_pca": (c.c_int32, [P, c.c_uint32, P, P]),
            "lpo_jacobi_svd2": (c.c_int32, [P, P]),
            "lpo_kdtree_positions": (c.c_int32, [P, c.c_uint32, P]),
            "lpo_glibc_rand": (c.c_int32, [c.c_uint64, c.c_uint32, P]),
            "lpo_cluster_objects": (c.c_int32, [P, P, c.c_uint32, c.c_uint32, P, P, P, P, P, P]),
            "lpo_debug_nth": (c.c_int32, [P, c.c_uint32, c.c_uint32, c.c_int32, c.c_int32, P]),
            "lpo_process_scan": (c.c_int32, [P, P, c.c_int, P]),
        }
        for k, (r, a) in sig.items():
            f = getattr(o, k)
            f.restype, f.argtypes = r, a
        _oracle = o
    return _oracle


def o_debug_sort(xy, variant):
    a = np.ascontiguousarray(xy, np.float64)
    out = np.zeros(len(a), np.int32)
    assert oracle().lpo_debug_sort(ptr(a), len(a), variant, ptr(out)) == 0
    return out


def have_ref():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        r = ctypes.CDLL(REF_PATH)
        P, c = ctypes.c_void_p, ctypes
        sig = {
            "lpr_segment": (c.c_int32, [P, P, c.c_uint32, P, P, P]),
            "lpr_noise_remove": (c.c_int32, [P, c.c_uint32, c.c_uint32, P, P]),
            "lpr_cluster": (c.c_int32, [P, c.c_uint32, c.c_uint32, P, P]),
            "lpr_convex_hull": (c.c_int32, [P, c.c_uint32, P, P]),
            "lpr_antipodal_pairs": (c.c_int32, [P, c.c_uint32, P, c.c_uint32, P]),
            "lpr_bounding_box_rotating_calipers": (c.c_int32, [P, c.c_uint32, P]),
            "lpr_bounding_box_pca": (c.c_int32, [P, c.c_uint32, P]),
            "lpr_process_scan": (c.c_int32, [P, P, P]),
            "lpr_add_ring_info": (c.c_int32, [P, c.c_uint32, P]),
        }
        for k, (rr, a) in sig.items():
            f = getattr(r, k)
            f.restype, f.argtypes = rr, a
        _ref = r
    return _ref


# ---------------------------------------------------------------------------- synthetic scans
synth_shape = lp.synth_shape  # the package's seeded generator (liblp_synth.so)
synth_scan = lp.synth_scan


# ------------------------------------------------------------------------------------------ I/O
def read_pcd(path):
    """Binary PCD v0.7 with FIELDS x y z intensity (the reference's data/*.pcd)."""
    with open(path, "rb") as f:
        data = f.read()
    head_end = data.index(b"DATA binary\n") + len(b"DATA binary\n")
    header = data[:head_end].decode()
    n = int(header.split("POINTS ")[1].split("\n")[0])
    return np.frombuffer(data[head_end:head_end + 16 * n], dtype=np.float32).reshape(n, 4).copy()


# --------------------------------------------------------------------------------- oracle calls
def o_ring(xyzi, first_ring=63, libm=LIBM_CR):
    oracle().lpo_set_libm_mode(libm)
    out = np.zeros(len(xyzi), np.uint16)
    oracle().lpo_add_ring_info(ptr(xyzi), len(xyzi), first_ring, ptr(out))
    return out


def o_segment(xyzi, ring, cfg, libm=LIBM_CR, image=False):
    oracle().lpo_set_libm_mode(libm)
    lab = np.zeros(len(xyzi), np.uint32)
    img = np.zeros((cfg.image_height, cfg.image_width, 3), np.uint8) if image else None
    st = oracle().lpo_segment(ptr(xyzi), ptr(ring), len(xyzi), ctypes.byref(cfg), ptr(lab), ptr(img))
    assert st == 0, st
    return (lab, img) if image else lab


def o_noise(pts, cfg, mode=DROR_KDTREE):
    a = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(a), np.uint8)
    st = oracle().lpo_noise_remove(ptr(a), a.shape[1], len(a), ctypes.byref(cfg), mode, ptr(out))
    assert st == 0, st
    return out


def o_cluster(pts, cfg, libm=LIBM_CR):
    oracle().lpo_set_libm_mode(libm)
    a = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(a), np.int32)
    st = oracle().lpo_cluster(ptr(a), a.shape[1], len(a), ctypes.byref(cfg), ptr(out))
    if st == lp.LP_ERR_CAPACITY:
        raise OverflowError("voxel capacity")
    assert st == 0, st
    return out


def o_hull(xy, ties=TIES_LIBSTDCXX):
    a = np.ascontiguousarray(xy, np.float64)
    out = np.zeros(len(a) + 1, np.int32)
    n = ctypes.c_uint32()
    oracle().lpo_set_hull_ties(ties)
    oracle().lpo_convex_hull(ptr(a), len(a), ptr(out), ctypes.byref(n))
    return out[: n.value].copy()


def o_calipers(hp):
    a = np.ascontiguousarray(hp, np.float64)
    b = lp.BoundingBox()
    oracle().lpo_bounding_box_rotating_calipers(ptr(a), len(a), ctypes.byref(b))
    return b


def o_pca(hp):
    a = np.ascontiguousarray(hp, np.float64)
    b = lp.BoundingBox()
    cov = np.zeros(3, np.float64)
    oracle().lpo_bounding_box_pca(ptr(a), len(a), ctypes.byref(b), ptr(cov))
    return b, cov


def o_svd2(a):
    """V (2x2) of the oracle's restatement of Eigen's JacobiSVD, or None for an invalid input."""
    m = np.ascontiguousarray(a, np.float64).reshape(4)
    v = np.zeros(4, np.float64)
    return v.reshape(2, 2) if oracle().lpo_jacobi_svd2(ptr(m), ptr(v)) == 0 else None


def o_kdtree_positions(xyz):
    """The reference kd-tree's points by node position (std::nth_element build), n x 3 float32."""
    a = np.ascontiguousarray(np.asarray(xyz, np.float32)[:, :3])
    out = np.zeros_like(a)
    oracle().lpo_kdtree_positions(ptr(a), len(a), ptr(out))
    return out


def o_debug_nth(v, nth, restated, depth_override=-1):
    a = np.ascontiguousarray(v, np.float32)
    out = np.zeros(len(a), np.int32)
    oracle().lpo_debug_nth(ptr(a), len(a), nth, int(restated), depth_override, ptr(out))
    return out


def o_glibc_rand(skip, count):
    out = np.zeros(count, np.int32)
    oracle().lpo_glibc_rand(skip, count, ptr(out))
    return out


def o_cluster_objects(cloud, result, vehicle_gates=False, rand_draws=0):
    """The oracle's restatement of the processor's per-cluster loop (processor.cpp:609-797)."""
    a = np.ascontiguousarray(np.asarray(cloud, np.float32)[:, :4])
    lab = np.ascontiguousarray(result.cluster_labels, np.int32)
    K = int(result.n_clusters)
    hoff = np.ascontiguousarray(result.hull_offsets[: K + 1], np.uint32)
    hidx = np.ascontiguousarray(result.hull_indices, np.int32)
    zmin = np.ascontiguousarray(result.z_min[:K], np.float32)
    zmax = np.ascontiguousarray(result.z_max[:K], np.float32)
    cfg = lp.ObjectConfig(1 if vehicle_gates else 0, 0, rand_draws)
    out, bufs = lp.object_buffers(len(a), K, hoff)
    st = oracle().lpo_cluster_objects(ptr(a), ptr(lab), len(a), K, ptr(hoff), ptr(hidx), ptr(zmin), ptr(zmax),
                                      ctypes.byref(cfg), ctypes.byref(out))
    assert st == 0, st
    return lp.ClusterObjects(bufs[0][: out.n_clustered].copy(), bufs[1][:K].copy(), list(bufs[2])[:K],
                             bufs[3].copy(), bufs[4][: out.n_marker_points].copy())


def o_antipodal(hp):
    a = np.ascontiguousarray(hp, np.float64)
    cap = 4 * len(a) + 8
    out = np.zeros((cap, 2), np.int32)
    n = ctypes.c_uint32()
    oracle().lpo_antipodal_pairs(ptr(a), len(a), ptr(out), cap, ctypes.byref(n))
    return out[: n.value].copy()


def o_process(xyzi, ring, seg_cfg, pipeline, libm=LIBM_CR, dror_mode=DROR_KDTREE, ties=TIES_LIBSTDCXX):
    oracle().lpo_set_libm_mode(libm)
    oracle().lpo_set_hull_ties(ties)
    b = lp.ResultBuffers(len(xyzi))
    scan = lp.ScanInput(xyzi.ctypes.data, None if ring is None else ring.ctypes.data, len(xyzi), seg_cfg)
    st = oracle().lpo_process_scan(ctypes.byref(pipeline), ctypes.byref(scan), dror_mode, ctypes.byref(b.out))
    assert st == 0, st
    return b.result()


# ------------------------------------------------------------------------------ reference calls
def r_segment(xyzi, ring, cfg, image=False):
    lab = np.zeros(len(xyzi), np.uint32)
    img = np.zeros((cfg.image_height, cfg.image_width, 3), np.uint8) if image else None
    st = ref().lpr_segment(ptr(xyzi), ptr(ring), len(xyzi), ctypes.byref(cfg), ptr(lab), ptr(img))
    assert st == 0, st
    return (lab, img) if image else lab


def r_ring(xyzi):
    """Ring indices from the reference's own Dataloader::addRingInfo (start ring 63)."""
    a = np.ascontiguousarray(xyzi, np.float32)
    out = np.zeros(len(a), np.uint16)
    assert ref().lpr_add_ring_info(ptr(a), len(a), ptr(out)) == 0
    return out


def r_noise(pts, cfg):
    a = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(a), np.uint8)
    assert ref().lpr_noise_remove(ptr(a), a.shape[1], len(a), ctypes.byref(cfg), ptr(out)) == 0
    return out


def r_cluster(pts, cfg):
    a = np.ascontiguousarray(pts, np.float32)
    out = np.zeros(len(a), np.int32)
    st = ref().lpr_cluster(ptr(a), a.shape[1], len(a), ctypes.byref(cfg), ptr(out))
    if st == lp.LP_ERR_CAPACITY:
        raise OverflowError("voxel capacity")
    assert st == 0
    return out


def r_hull(xy):
    a = np.ascontiguousarray(xy, np.float64)
    out = np.zeros(len(a) + 1, np.int32)
    n = ctypes.c_uint32()
    ref().lpr_convex_hull(ptr(a), len(a), ptr(out), ctypes.byref(n))
    return out[: n.value].copy()


def r_calipers(hp):
    a = np.ascontiguousarray(hp, np.float64)
    b = lp.BoundingBox()
    ref().lpr_bounding_box_rotating_calipers(ptr(a), len(a), ctypes.byref(b))
    return b


def r_pca(hp):
    a = np.ascontiguousarray(hp, np.float64)
    b = lp.BoundingBox()
    ref().lpr_bounding_box_pca(ptr(a), len(a), ctypes.byref(b))
    return b


def r_antipodal(hp):
    a = np.ascontiguousarray(hp, np.float64)
    cap = 4 * len(a) + 8
    out = np.zeros((cap, 2), np.int32)
    n = ctypes.c_uint32()
    ref().lpr_antipodal_pairs(ptr(a), len(a), ptr(out), cap, ctypes.byref(n))
    return out[: n.value].copy()


def r_process(xyzi, ring, seg_cfg, pipeline):
    b = lp.ResultBuffers(len(xyzi))
    scan = lp.ScanInput(xyzi.ctypes.data, None if ring is None else ring.ctypes.data, len(xyzi), seg_cfg)
    st = ref().lpr_process_scan(ctypes.byref(pipeline), ctypes.byref(scan), ctypes.byref(b.out))
    assert st == 0, st
    return b.result()


# --------------------------------------------------------------------------------- comparisons
def box_corner_set_close(b1, b2, tol=1e-4):
    """Corners of two boxes describe the same rectangle within tol: some one-to-one assignment of
    the corners (any order) keeps every pair within tol. All 24 assignments are tried; a greedy
    nearest-corner match would fail on boxes narrower than the tolerance, whose corners pair up
    ambiguously."""
    if bool(b1.is_valid) != bool(b2.is_valid):
        return False
    if not b1.is_valid:
        return True
    c1, c2 = b1.corners_array(), b2.corners_array()
    d = np.abs(c1[:, None, :] - c2[None, :, :]).max(axis=2)  # d[i, j]: corner i of b1 to corner j of b2
    return any(max(d[i, p[i]] for i in range(4)) <= tol for p in itertools.permutations(range(4)))


def boxes_identical(b1, b2):
    return (b1.is_valid == b2.is_valid and (not b1.is_valid or (
        np.array_equal(b1.corners_array(), b2.corners_array()) and b1.area == b2.area
        and b1.angle_rad == b2.angle_rad)))


def pca_boxes_equal(b1, b2):
    """PCA boxes computed by the same binary64 steps: validity, corners (in order) and area
    identical; the angle (binary64 atan2 of the axis, rounded to float) within one float ulp,
    since the device's and the host's atan2 may differ in the last binary64 bit."""
    if bool(b1.is_valid) != bool(b2.is_valid):
        return False
    if not b1.is_valid:
        return True
    ulp = float(np.spacing(np.float32(abs(b2.angle_rad))))
    return (np.array_equal(b1.corners_array(), b2.corners_array()) and b1.area == b2.area
            and abs(b1.angle_rad - b2.angle_rad) <= ulp)


def same_partition(a, b):
    """Two labelings describe the same partition (labels equal up to a bijection)."""
    if a.shape != b.shape:
        return False
    pairs = set(zip(a.tolist(), b.tolist()))
    fa = {}
    fb = {}
    for x, y in pairs:
        if fa.setdefault(x, y) != y or fb.setdefault(y, x) != x:
            return False
    return True
