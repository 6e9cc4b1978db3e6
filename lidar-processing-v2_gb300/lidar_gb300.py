"""Python host API for the GB300 LiDAR perception library (ctypes over liblp_gpu.so).

Mirrors the reference library's classes (lidar_processing_lib, YevgeniyEngineer/LiDAR-Processing-V2):

    Segmenter.segment(cloud)            segmenter.cpp:87-101   -> uint32 labels (UNKNOWN/GROUND/OBSTACLE)
    NoiseRemover.filter(points)         noise_remover.cpp:38-68 -> uint8 labels (VALID/NOISE)
    Clusterer.cluster(cloud)            clusterer.cpp:43-53    -> int32 labels (-1 = none)
    Polygonizer.convexHull(points)      polygonizer.cpp:33-91  -> int32 hull indices
    Polygonizer.boundingBoxRotatingCalipers / boundingBoxPrincipalComponentAnalysis
    add_ring_info(cloud)                dataloader.cpp:68-137  -> uint16 rings

and the batched pipeline (process_batch). Errors raise the exception type the reference throws for
the same condition (RuntimeError, OverflowError, ValueError). Every call runs CUDA kernels; the
library refuses to load, rather than falling back to the CPU, when its shared object is missing.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liblp_gpu.so")
SYNTH_PATH = os.path.join(_HERE, "liblp_synth.so")

LP_OK, LP_ERR_BAD_ARG, LP_ERR_CAPACITY, LP_ERR_TIMEOUT, LP_ERR_CUDA, LP_ERR_NO_DEVICE, LP_ERR_INTERNAL = range(7)
UNKNOWN, GROUND, OBSTACLE = 0, 1, 2
VALID, NOISE = 0, 1
INVALID_CLUSTER = -1


class SegmenterConfig(ctypes.Structure):
    """lp_segmenter_config == SegmenterConfiguration (segmenter.hpp:87-112)."""

    _fields_ = [
        ("elevation_up_deg", ctypes.c_float),
        ("elevation_down_deg", ctypes.c_float),
        ("image_width", ctypes.c_int32),
        ("image_height", ctypes.c_int32),
        ("assume_unorganized_cloud", ctypes.c_int32),
        ("grid_radial_spacing_m", ctypes.c_float),
        ("grid_slice_resolution_deg", ctypes.c_float),
        ("ground_height_threshold_m", ctypes.c_float),
        ("road_maximum_slope_m_per_m", ctypes.c_float),
        ("min_distance_m", ctypes.c_float),
        ("max_distance_m", ctypes.c_float),
        ("sensor_height_m", ctypes.c_float),
        ("kernel_threshold_distance_m", ctypes.c_float),
        ("amplification_factor", ctypes.c_float),
        ("z_min_m", ctypes.c_float),
        ("z_max_m", ctypes.c_float),
    ]

    @classmethod
    def default(cls, **kw):
        c = cls(2.0, -24.8, 2048, 64, 0, 2.0, 1.0, 0.2, 0.2, 2.0, 100.0, 1.73, 1.0, 5.0, -3.0, 4.0)
        for k, v in kw.items():
            setattr(c, k, v)
        return c


class NoiseRemoverConfig(ctypes.Structure):
    """lp_noise_remover_config == NoiseRemoverConfiguration (noise_remover.hpp:41-54)."""

    _fields_ = [
        ("radius_multiplier_m_per_m", ctypes.c_float),
        ("min_search_radius_m", ctypes.c_float),
        ("min_neighbours", ctypes.c_uint32),
    ]

    @classmethod
    def default(cls, **kw):
        c = cls(0.02, 0.1, 4)
        for k, v in kw.items():
            setattr(c, k, v)
        return c


class ClustererConfig(ctypes.Structure):
    """lp_clusterer_config == ClustererConfiguration (clusterer.hpp:61-68)."""

    _fields_ = [
        ("voxel_grid_range_resolution_m", ctypes.c_float),
        ("voxel_grid_azimuth_resolution_deg", ctypes.c_float),
        ("voxel_grid_elevation_resolution_deg", ctypes.c_float),
        ("min_cluster_size", ctypes.c_uint32),
    ]

    @classmethod
    def default(cls, **kw):
        c = cls(0.4, 1.0, 1.5, 3)
        for k, v in kw.items():
            setattr(c, k, v)
        return c

    @classmethod
    def processor(cls):
        """The processor node's YAML values (processor.param.yaml:31-35): elevation 3.0 deg."""
        return cls(0.4, 1.0, 3.0, 3)


class BoundingBox(ctypes.Structure):
    """lp_bounding_box == BoundingBox (polygonizer.hpp:75-81)."""

    _fields_ = [
        ("corners", (ctypes.c_double * 2) * 4),
        ("area", ctypes.c_float),
        ("angle_rad", ctypes.c_float),
        ("is_valid", ctypes.c_int32),
    ]

    def corners_array(self):
        return np.array([[self.corners[k][0], self.corners[k][1]] for k in range(4)])


class PipelineConfig(ctypes.Structure):
    _fields_ = [
        ("cluster", ClustererConfig),
        ("noise", NoiseRemoverConfig),
        ("enable_noise_removal", ctypes.c_int32),
        ("compute_ring", ctypes.c_int32),
        ("first_ring", ctypes.c_uint16),
        ("reserved0", ctypes.c_uint16),
        ("compute_obb", ctypes.c_int32),
    ]

    @classmethod
    def default(cls, **kw):
        """Processor settings; first_ring 0 means image_height - 1 (63 for the 64-ring sensor,
        the reference's hard-coded start ring, dataloader.cpp:87)."""
        c = cls(ClustererConfig.processor(), NoiseRemoverConfig.default(), 0, 0, 0, 0, 1)
        for k, v in kw.items():
            setattr(c, k, v)
        return c


class ScanInput(ctypes.Structure):
    _fields_ = [
        ("xyzi", ctypes.c_void_p),
        ("ring", ctypes.c_void_p),
        ("n", ctypes.c_uint32),
        ("seg", SegmenterConfig),
    ]


class ScanOutput(ctypes.Structure):
    _fields_ = [
        ("noise_labels", ctypes.c_void_p),
        ("seg_labels", ctypes.c_void_p),
        ("cluster_labels", ctypes.c_void_p),
        ("cluster_capacity", ctypes.c_uint32),
        ("hull_capacity", ctypes.c_uint32),
        ("hull_offsets", ctypes.c_void_p),
        ("hull_indices", ctypes.c_void_p),
        ("z_min", ctypes.c_void_p),
        ("z_max", ctypes.c_void_p),
        ("obb_calipers", ctypes.c_void_p),
        ("obb_pca", ctypes.c_void_p),
        ("n_obstacles", ctypes.c_uint32),
        ("n_clusters", ctypes.c_uint32),
        ("n_hull_indices", ctypes.c_uint32),
        ("status", ctypes.c_int32),
    ]


def ptr(a):
    """ctypes void pointer of a contiguous numpy array (None passes NULL)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class ScanResult:
    noise_labels: np.ndarray
    seg_labels: np.ndarray
    cluster_labels: np.ndarray
    n_obstacles: int
    n_clusters: int
    hull_offsets: np.ndarray
    hull_indices: np.ndarray
    z_min: np.ndarray
    z_max: np.ndarray
    obb_calipers: list
    obb_pca: list

    def hull(self, k):
        return self.hull_indices[self.hull_offsets[k]:self.hull_offsets[k + 1]]


class _PinnedBlock:
    """One lp_host_alloc allocation, freed when the last array viewing it is gone."""

    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        check(library().lp_host_alloc(max(1, int(nbytes)), ctypes.byref(p)))
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def __del__(self):
        try:
            library().lp_host_free(ctypes.c_void_p(self.ptr))
        except Exception:
            pass


def pinned_empty(shape, dtype):
    """numpy array in page-locked host memory (lp_host_alloc); contents undefined."""
    dt = np.dtype(dtype)
    count = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    blk = _PinnedBlock(count * dt.itemsize)
    buf = (ctypes.c_char * max(1, blk.nbytes)).from_address(blk.ptr)
    buf._owner = blk  # the array's base is `buf`, which keeps the allocation alive
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


def pinned_copy(a):
    """Page-locked copy of a numpy array."""
    out = pinned_empty(a.shape, a.dtype)
    out[...] = a
    return out


class ResultBuffers:
    """Host result buffers for one scan, in the layout lp_scan_output points at. With pinned=True
    they live in page-locked memory (lp_host_alloc) and can be reused call after call."""

    def __init__(self, n, cluster_capacity=None, hull_capacity=None, pinned=False):
        cc = cluster_capacity if cluster_capacity is not None else max(64, n // 3 + 1)
        hc = hull_capacity if hull_capacity is not None else max(256, n + cc)
        alloc = pinned_empty if pinned else (lambda shape, dt: np.zeros(shape, dt))
        self.noise = alloc(n, np.uint8)
        self.seg = alloc(n, np.uint32)
        self.cl = alloc(n, np.int32)
        self.hoff = alloc(cc + 1, np.uint32)
        self.hidx = alloc(hc, np.int32)
        self.zmin = alloc(cc, np.float32)
        self.zmax = alloc(cc, np.float32)
        if pinned:
            self._obb = alloc(2 * cc * ctypes.sizeof(BoundingBox), np.uint8)
            self.obb_c = (BoundingBox * cc).from_address(self._obb.ctypes.data)
            self.obb_p = (BoundingBox * cc).from_address(self._obb.ctypes.data + cc * ctypes.sizeof(BoundingBox))
        else:
            self.obb_c = (BoundingBox * cc)()
            self.obb_p = (BoundingBox * cc)()
        self.out = ScanOutput(ptr(self.noise), ptr(self.seg), ptr(self.cl), cc, hc, ptr(self.hoff),
                              ptr(self.hidx), ptr(self.zmin), ptr(self.zmax),
                              ctypes.cast(self.obb_c, ctypes.c_void_p), ctypes.cast(self.obb_p, ctypes.c_void_p),
                              0, 0, 0, 0)

    def result(self):
        k = self.out.n_clusters
        return ScanResult(self.noise.copy(), self.seg.copy(), self.cl.copy(), self.out.n_obstacles, k,
                          self.hoff[:k + 1].copy(), self.hidx[:self.out.n_hull_indices].copy(),
                          self.zmin[:k].copy(), self.zmax[:k].copy(),
                          [self.obb_c[i] for i in range(k)], [self.obb_p[i] for i in range(k)])


def _declare(lib):
    c = ctypes
    P = c.c_void_p
    sig = {
        "lp_context_create": (c.c_int32, [c.c_int32, c.POINTER(P)]),
        "lp_context_destroy": (None, [P]),
        "lp_status_string": (c.c_char_p, [c.c_int32]),
        "lp_last_error": (c.c_char_p, [P]),
        "lp_kernel_launch_count": (c.c_uint64, [P]),
        "lp_add_ring_info": (c.c_int32, [P, P, c.c_uint32, c.c_uint16, P]),
        "lp_split_clouds": (c.c_int32, [P, P, P, c.c_uint32, P, P, P, P]),
        "lp_cluster_objects": (c.c_int32, [P, P, P, c.c_uint32, c.c_uint32, P, P, P, P, P, P]),
        "lp_unpack_pointcloud2": (c.c_int32, [P, P, c.c_uint32, c.c_uint32, c.c_uint32, c.c_uint32, P, P, P]),
        "lp_segment": (c.c_int32, [P, P, P, c.c_uint32, P, P, P]),
        "lp_noise_remove": (c.c_int32, [P, P, c.c_uint32, c.c_uint32, P, P]),
        "lp_cluster": (c.c_int32, [P, P, c.c_uint32, c.c_uint32, P, P]),
        "lp_convex_hull": (c.c_int32, [P, P, c.c_uint32, P, P]),
        "lp_antipodal_pairs": (c.c_int32, [P, P, c.c_uint32, P, c.c_uint32, P]),
        "lp_bounding_box_rotating_calipers": (c.c_int32, [P, P, c.c_uint32, P]),
        "lp_bounding_box_pca": (c.c_int32, [P, P, c.c_uint32, P]),
        "lp_process_scan": (c.c_int32, [P, P, P, P]),
        "lp_process_batch": (c.c_int32, [P, P, P, P, c.c_uint32]),
        "lp_batch_create": (c.c_int32, [P, P, P, c.c_uint32, c.POINTER(P)]),
        "lp_batch_destroy": (None, [P, P]),
        "lp_batch_upload": (c.c_int32, [P, P]),
        "lp_batch_execute": (c.c_int32, [P, P]),
        "lp_batch_capture_graph": (c.c_int32, [P, P]),
        "lp_batch_download": (c.c_int32, [P, P, P]),
        "lp_context_synchronize": (c.c_int32, [P]),
        "lp_batch_points": (c.c_uint32, [P]),
        "lp_batch_device_bytes": (c.c_uint64, [P]),
        "lp_batch_time": (c.c_int32, [P, P, c.c_uint32, c.c_int32, c.POINTER(c.c_float)]),
        "lp_batch_profile": (c.c_int32, [P, P, P, c.c_uint32, P, c.c_uint32, c.POINTER(c.c_uint32)]),
        "lp_debug_math": (c.c_int32, [P, c.c_int32, P, P, c.c_uint32, P]),
        "lp_host_alloc": (c.c_int32, [c.c_uint64, c.POINTER(P)]),
        "lp_host_free": (None, [P]),
        "lp_debug_math_sweep": (c.c_int32, [P, c.c_int32, c.c_uint64, c.c_uint64, P, P]),
        "lp_server_config_default": (None, [P]),
        "lp_server_create": (c.c_int32, [c.c_int32, P, P, c.POINTER(P)]),
        "lp_server_submit": (c.c_int32, [P, P, P, c.c_uint64]),
        "lp_server_poll": (c.c_int32, [P, P, c.c_uint32, c.POINTER(c.c_uint32), c.c_uint32]),
        "lp_server_stats_get": (c.c_int32, [P, P]),
        "lp_server_destroy": (None, [P]),
        "lp_server_hold": (c.c_int32, [P, c.c_int32]),
        "lp_tuning_default": (None, [P]),
        "lp_tuning_validate": (c.c_int32, [P]),
        "lp_tuning_key_of": (c.c_int32, [P, c.c_uint32, P]),
        "lp_tuning_table_create": (c.c_int32, [c.POINTER(P)]),
        "lp_tuning_table_destroy": (None, [P]),
        "lp_tuning_table_set": (c.c_int32, [P, P, P, c.c_float]),
        "lp_tuning_table_get": (c.c_int32, [P, P, P, c.POINTER(c.c_float)]),
        "lp_tuning_table_size": (c.c_uint32, [P]),
        "lp_tuning_table_save": (c.c_int32, [P, c.c_char_p]),
        "lp_tuning_table_load": (c.c_int32, [P, c.c_char_p]),
        "lp_context_set_tuning_table": (c.c_int32, [P, P]),
        "lp_batch_create_tuned": (c.c_int32, [P, P, P, c.c_uint32, P, c.POINTER(P)]),
        "lp_batch_get_tuning": (c.c_int32, [P, P]),
        "lp_autotune": (c.c_int32, [P, P, P, c.c_uint32, c.c_uint32, P, P, P, P, P, c.c_uint32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


_lib = None


def library():
    """Load liblp_gpu.so (built in-tree by __graft_entry__.build()). Raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"liblp_gpu.so not built at {LIB_PATH}; run __graft_entry__.build()")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


class LidarError(RuntimeError):
    pass


def check(status, ctx=None):
    if status == LP_OK:
        return
    lib = library()
    msg = lib.lp_status_string(status).decode()
    if ctx is not None:
        detail = lib.lp_last_error(ctx.handle)
        if detail:
            msg += ": " + detail.decode()
    if status == LP_ERR_CAPACITY:
        raise OverflowError(msg)
    if status == LP_ERR_BAD_ARG:
        raise ValueError(msg)
    raise LidarError(msg)


class Context:
    """One device context (device buffers, stream). Not thread-safe, like the reference objects."""

    def __init__(self, device=0):
        lib = library()
        h = ctypes.c_void_p()
        check(lib.lp_context_create(device, ctypes.byref(h)))
        self.handle = h

    def close(self):
        if self.handle:
            library().lp_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tuning_table(self, table):
        """Batches created in this context afterwards take their bucket's entry of `table` (a TuningTable;
        None clears)."""
        check(library().lp_context_set_tuning_table(self.handle, table.handle if table is not None else None), self)

    @property
    def launches(self):
        return int(library().lp_kernel_launch_count(self.handle))


def _xyzi(cloud):
    a = np.ascontiguousarray(cloud, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] not in (3, 4):
        raise ValueError("cloud must be N x 3 or N x 4 float32")
    if a.shape[1] == 3:
        a = np.ascontiguousarray(np.concatenate([a, np.zeros((len(a), 1), np.float32)], axis=1))
    return a


def add_ring_info(ctx, cloud, first_ring=63):
    a = _xyzi(cloud)
    out = np.zeros(len(a), np.uint16)
    check(library().lp_add_ring_info(ctx.handle, ptr(a), len(a), first_ring, ptr(out)), ctx)
    return out


# lp_xyzrgb: pcl::PointXYZRGB's position and colour
XYZRGB = np.dtype([("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("r", "u1"), ("g", "u1"), ("b", "u1"), ("a", "u1")])


NO_FIELD = 0xFFFFFFFF


def unpack_pointcloud2(ctx, data, width, height, point_step, row_step, x=0, y=4, z=8, intensity=NO_FIELD,
                       ring=NO_FIELD):
    """sensor_msgs/PointCloud2 bytes -> (xyzi float32 (n, 4), ring uint16 (n,) or None), as the
    processor's convert<PointT> (processor.cpp:42-179); arguments are the message's layout and the
    byte offsets of its fields (intensity / ring NO_FIELD when absent)."""
    buf = np.ascontiguousarray(np.frombuffer(data, np.uint8) if not isinstance(data, np.ndarray) else data.view(np.uint8).reshape(-1))
    n = width * height
    xyzi = np.zeros((n, 4), np.float32)
    rg = np.zeros(n, np.uint16) if ring != NO_FIELD else None
    offs = np.array([x, y, z, intensity, ring], np.uint32)
    check(library().lp_unpack_pointcloud2(ctx.handle, ptr(buf), width, height, point_step, row_step, ptr(offs),
                                          ptr(xyzi), None if rg is None else ptr(rg)), ctx)
    return xyzi, rg


def split_clouds(ctx, cloud, labels):
    """The processor's ground, obstacle and unsegmented clouds (processor.cpp:558-579): the points
    of each segmentation label class in input order, coloured (124, 252, 0), (200, 0, 0) and
    (255, 255, 0). Returns three XYZRGB structured arrays."""
    a = _xyzi(cloud)
    lab = np.ascontiguousarray(labels, np.uint32)
    if len(lab) != len(a):
        raise ValueError("one label per point")
    outs = [np.zeros(len(a), XYZRGB) for _ in range(3)]
    counts = np.zeros(3, np.uint32)
    check(library().lp_split_clouds(ctx.handle, ptr(a), ptr(lab), len(a), ptr(outs[0]), ptr(outs[1]), ptr(outs[2]),
                                    ptr(counts)), ctx)
    return tuple(o[:k] for o, k in zip(outs, counts))


class ObjectConfig(ctypes.Structure):
    """lp_object_config: the vehicle gates on or off and the std::rand() draws made before."""

    _fields_ = [("vehicle_gates", ctypes.c_int32), ("reserved", ctypes.c_uint32), ("rand_draws", ctypes.c_uint64)]


class ObjectOutput(ctypes.Structure):
    _fields_ = [
        ("clustered_cloud", ctypes.c_void_p),
        ("vehicle_class", ctypes.c_void_p),
        ("gate_boxes", ctypes.c_void_p),
        ("marker_offsets", ctypes.c_void_p),
        ("marker_points", ctypes.c_void_p),
        ("marker_capacity", ctypes.c_uint32),
        ("n_clustered", ctypes.c_uint32),
        ("n_marker_points", ctypes.c_uint32),
    ]


class ClusterObjects:
    """The processor's per-cluster products of one scan (processor.cpp:609-797): the clustered cloud
    (XYZRGB records by label, colours from std::rand()), the vehicle class per cluster (-1 when not
    boxed), the gate's calipers boxes, and the boundary marker points (n x 3 float64, offsets per
    cluster)."""

    def __init__(self, cloud, vehicle_class, gate_boxes, marker_offsets, marker_points):
        self.cloud = cloud
        self.vehicle_class = vehicle_class
        self.gate_boxes = gate_boxes
        self.marker_offsets = marker_offsets
        self.marker_points = marker_points


def object_buffers(n, n_clusters, hull_offsets):
    """Output buffers of lp_cluster_objects sized for n points and the given hulls."""
    K = int(n_clusters)
    mcap = 6 * (int(hull_offsets[K]) + 4 * K) if K else 0
    bufs = (np.zeros(max(n, 1), XYZRGB), np.full(max(K, 1), -7, np.int32), (BoundingBox * max(K, 1))(),
            np.zeros(K + 1, np.uint32), np.zeros((max(mcap, 1), 3), np.float64))
    out = ObjectOutput(ptr(bufs[0]), ptr(bufs[1]), ctypes.cast(bufs[2], ctypes.c_void_p).value, ptr(bufs[3]),
                       ptr(bufs[4]), mcap, 0, 0)
    return out, bufs


def cluster_objects(ctx, cloud, result, vehicle_gates=False, rand_draws=0):
    """lp_cluster_objects over one scan's pipeline result (cluster labels, hulls, z ranges)."""
    a = _xyzi(cloud)
    lab = np.ascontiguousarray(result.cluster_labels, np.int32)
    K = int(result.n_clusters)
    hoff = np.ascontiguousarray(result.hull_offsets[: K + 1], np.uint32)
    hidx = np.ascontiguousarray(result.hull_indices, np.int32)
    zmin = np.ascontiguousarray(result.z_min[:K], np.float32)
    zmax = np.ascontiguousarray(result.z_max[:K], np.float32)
    cfg = ObjectConfig(1 if vehicle_gates else 0, 0, rand_draws)
    out, bufs = object_buffers(len(a), K, hoff)
    check(library().lp_cluster_objects(ctx.handle, ptr(a), ptr(lab), len(a), K, ptr(hoff), ptr(hidx), ptr(zmin),
                                       ptr(zmax), ctypes.byref(cfg), ctypes.byref(out)), ctx)
    return ClusterObjects(bufs[0][: out.n_clustered].copy(), bufs[1][:K].copy(), list(bufs[2])[:K],
                          bufs[3].copy(), bufs[4][: out.n_marker_points].copy())


class Segmenter:
    """Segmenter (segmenter.hpp:131-262): config() then segment(cloud[, ring]) -> labels."""

    def __init__(self, ctx, config=None):
        self.ctx = ctx
        self._config = config or SegmenterConfig.default()
        self._image = None

    def config(self, cfg=None):
        if cfg is not None:
            self._config = cfg
        return self._config

    def segment(self, cloud, ring=None, want_image=False):
        a = _xyzi(cloud)
        labels = np.zeros(len(a), np.uint32)
        img = np.zeros((self._config.image_height, self._config.image_width, 3), np.uint8) if want_image else None
        r = None if ring is None else np.ascontiguousarray(ring, dtype=np.uint16)
        check(library().lp_segment(self.ctx.handle, ptr(a), ptr(r), len(a), ctypes.byref(self._config),
                                   ptr(labels), ptr(img)), self.ctx)
        self._image = img
        return labels

    def image(self):
        return self._image


# ------------------------------------------------------------------ seeded synthetic scans
_synth = None


def _synth_lib():
    """liblp_synth.so: the seeded synthetic scan generator the benchmarks and tests draw from
    (spinning 32/64/128-ring sensor, ray-cast ground, boxes, cylinders, wall; workloads 1-5)."""
    global _synth
    if _synth is None:
        s = ctypes.CDLL(SYNTH_PATH)
        P = ctypes.c_void_p
        s.lp_synth_capacity.restype = ctypes.c_uint32
        s.lp_synth_capacity.argtypes = [ctypes.c_int32, ctypes.c_int32]
        s.lp_synth_scan.restype = ctypes.c_uint32
        s.lp_synth_scan.argtypes = [ctypes.c_int32, ctypes.c_int32, P, P, ctypes.c_uint32]
        s.lp_synth_shape.restype = None
        s.lp_synth_shape.argtypes = [ctypes.c_int32, ctypes.c_int32, P, P, P, P]
        _synth = s
    return _synth


def synth_shape(workload, scan):
    """(rings, azimuth bins, elevation up deg, elevation down deg) of a seeded synthetic scan."""
    r, w, up, dn = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_float(), ctypes.c_float()
    _synth_lib().lp_synth_shape(workload, scan, ctypes.byref(r), ctypes.byref(w), ctypes.byref(up), ctypes.byref(dn))
    return r.value, w.value, up.value, dn.value


def synth_scan(workload, scan):
    """(xyzi float32 N x 4, true ring uint16, SegmenterConfig) of seeded synthetic scan `scan` of
    workload 1-5 (seed 1000 * workload + scan)."""
    cap = _synth_lib().lp_synth_capacity(workload, scan)
    x = np.zeros((cap, 4), np.float32)
    r = np.zeros(cap, np.uint16)
    n = _synth_lib().lp_synth_scan(workload, scan, ptr(x), ptr(r), cap)
    rings, bins, up, dn = synth_shape(workload, scan)
    cfg = SegmenterConfig.default(image_height=rings, image_width=bins, elevation_up_deg=up, elevation_down_deg=dn)
    return np.ascontiguousarray(x[:n]), np.ascontiguousarray(r[:n]), cfg


def debug_kdtree(ctx, xyz, config=None):
    """The outlier filter's device kd-tree for the cloud xyz: per node position x, y, z (float32,
    n x 3) and subtree sizes (uint32, n), as lp_debug_kdtree returns them."""
    a = np.ascontiguousarray(xyz, np.float32)
    n = len(a)
    out = np.zeros((n, 4), np.float32)
    cfg = config or NoiseRemoverConfig.default()
    lib = library()
    lib.lp_debug_kdtree.restype = ctypes.c_int32
    lib.lp_debug_kdtree.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_void_p, ctypes.c_void_p]
    check(lib.lp_debug_kdtree(ctx.handle, ptr(a), a.shape[1], n, ctypes.byref(cfg), ptr(out)), ctx)
    return np.ascontiguousarray(out[:, :3]), out[:, 3].view(np.uint32).copy()


class NoiseRemover:
    """NoiseRemover (noise_remover.hpp:56-86): filter(points) -> VALID/NOISE per point."""

    def __init__(self, ctx, config=None):
        self.ctx = ctx
        self._config = config or NoiseRemoverConfig.default()

    def config(self, cfg=None):
        if cfg is not None:
            self._config = cfg
        return self._config

    def filter(self, points):
        a = np.ascontiguousarray(points, dtype=np.float32)
        out = np.zeros(len(a), np.uint8)
        check(library().lp_noise_remove(self.ctx.handle, ptr(a), a.shape[1], len(a), ctypes.byref(self._config),
                                        ptr(out)), self.ctx)
        return out


class Clusterer:
    """Clusterer (clusterer.hpp:70-175): cluster(cloud) -> int32 labels."""

    def __init__(self, ctx, config=None):
        self.ctx = ctx
        self._config = config or ClustererConfig.default()

    def config(self, cfg=None):
        if cfg is not None:
            self._config = cfg
        return self._config

    def cluster(self, cloud):
        a = np.ascontiguousarray(cloud, dtype=np.float32)
        out = np.zeros(len(a), np.int32)
        check(library().lp_cluster(self.ctx.handle, ptr(a), a.shape[1], len(a), ctypes.byref(self._config),
                                   ptr(out)), self.ctx)
        return out


class Polygonizer:
    """Polygonizer (polygonizer.hpp:85-150)."""

    def __init__(self, ctx):
        self.ctx = ctx

    def convexHull(self, points):
        a = np.ascontiguousarray(points, dtype=np.float64)
        out = np.zeros(len(a) + 1, np.int32)
        n = ctypes.c_uint32()
        check(library().lp_convex_hull(self.ctx.handle, ptr(a), len(a), ptr(out), ctypes.byref(n)), self.ctx)
        return out[: n.value].copy()

    def findAntipodalPairsOfConvexHull(self, hull_points):
        a = np.ascontiguousarray(hull_points, dtype=np.float64)
        cap = 4 * len(a) + 8
        out = np.zeros((cap, 2), np.int32)
        n = ctypes.c_uint32()
        check(library().lp_antipodal_pairs(self.ctx.handle, ptr(a), len(a), ptr(out), cap, ctypes.byref(n)), self.ctx)
        return out[: n.value].copy()

    def boundingBoxRotatingCalipers(self, hull_points):
        a = np.ascontiguousarray(hull_points, dtype=np.float64)
        b = BoundingBox()
        check(library().lp_bounding_box_rotating_calipers(self.ctx.handle, ptr(a), len(a), ctypes.byref(b)), self.ctx)
        return b

    def boundingBoxPrincipalComponentAnalysis(self, hull_points):
        a = np.ascontiguousarray(hull_points, dtype=np.float64)
        b = BoundingBox()
        check(library().lp_bounding_box_pca(self.ctx.handle, ptr(a), len(a), ctypes.byref(b)), self.ctx)
        return b


class Tuning(ctypes.Structure):
    """lp_tuning: a batch's split into concurrent parts and its launch shapes (results never
    depend on it)."""
    _fields_ = [("parts", ctypes.c_uint32), ("balance_parts", ctypes.c_uint32), ("hull_cta_min", ctypes.c_uint32),
                ("hull_ctas_per_sm", ctypes.c_uint32), ("cell_ctas_per_sm", ctypes.c_uint32),
                ("jcp_ctas_per_sm", ctypes.c_uint32)]

    @staticmethod
    def default(**kw):
        t = Tuning()
        library().lp_tuning_default(ctypes.byref(t))
        for k, v in kw.items():
            setattr(t, k, v)
        return t

    def valid(self):
        return library().lp_tuning_validate(ctypes.byref(self)) == LP_OK

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class TuningKey(ctypes.Structure):
    _fields_ = [("scans_class", ctypes.c_uint32), ("ring_class", ctypes.c_uint32), ("azimuth_class", ctypes.c_uint32)]

    def as_tuple(self):
        return (int(self.scans_class), int(self.ring_class), int(self.azimuth_class))


class AutotuneReport(ctypes.Structure):
    _fields_ = [("trials", ctypes.c_uint32), ("start_ms", ctypes.c_float), ("best_ms", ctypes.c_float)]


def _scan_inputs(scans, seg_configs=None, rings=None):
    """(ScanInput array, arrays kept alive) for a list of clouds."""
    n = len(scans)
    arrs = [_xyzi(s) for s in scans]
    rs = [None if (rings is None or rings[i] is None) else np.ascontiguousarray(rings[i], np.uint16) for i in range(n)]
    cfgs = seg_configs or [SegmenterConfig.default() for _ in range(n)]
    ins = (ScanInput * n)()
    for i in range(n):
        ins[i] = ScanInput(arrs[i].ctypes.data, None if rs[i] is None else rs[i].ctypes.data, len(arrs[i]), cfgs[i])
    return ins, (arrs, rs)


def tuning_key(scans, seg_configs=None):
    ins, keep = _scan_inputs(scans, seg_configs)
    k = TuningKey()
    check(library().lp_tuning_key_of(ins, len(scans), ctypes.byref(k)))
    return k


class TuningTable:
    """Host table bucket -> tuning (lp_tuning_table)."""

    def __init__(self):
        h = ctypes.c_void_p()
        check(library().lp_tuning_table_create(ctypes.byref(h)))
        self.handle = h

    def set(self, key, tuning, ms=0.0):
        check(library().lp_tuning_table_set(self.handle, ctypes.byref(key), ctypes.byref(tuning), ms))

    def get(self, key):
        """(found, Tuning, ms): the defaults and found=False when the bucket has no entry."""
        t = Tuning()
        ms = ctypes.c_float()
        found = library().lp_tuning_table_get(self.handle, ctypes.byref(key), ctypes.byref(t), ctypes.byref(ms))
        return bool(found), t, float(ms.value)

    def __len__(self):
        return int(library().lp_tuning_table_size(self.handle))

    def save(self, path):
        check(library().lp_tuning_table_save(self.handle, os.fsencode(path)))

    def load(self, path):
        check(library().lp_tuning_table_load(self.handle, os.fsencode(path)))

    def close(self):
        if self.handle:
            library().lp_tuning_table_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(ctx, scans, pipeline=None, seg_configs=None, rings=None, iters=5, table=None, trial_cap=64):
    """lp_autotune: (best Tuning, report dict with the timed candidates) for these scans; the choice is
    stored in `table` (a TuningTable) under the scans' bucket when one is given."""
    pipeline = pipeline or PipelineConfig.default()
    ins, keep = _scan_inputs(scans, seg_configs, rings)
    best = Tuning()
    rep = AutotuneReport()
    tms = np.zeros(trial_cap, np.float32)
    tcf = (Tuning * trial_cap)()
    check(library().lp_autotune(ctx.handle, ctypes.byref(pipeline), ins, len(scans), iters,
                                table.handle if table is not None else None, ctypes.byref(best), ctypes.byref(rep),
                                ptr(tms), tcf, trial_cap), ctx)
    k = min(rep.trials, trial_cap)
    return best, {"trials": int(rep.trials), "start_ms": float(rep.start_ms), "best_ms": float(rep.best_ms),
                  "candidates": [(tcf[i].as_dict(), float(tms[i])) for i in range(k)]}


class PreparedBatch:
    """Scans uploaded once to HBM; execute() re-runs the pipeline on the device-resident inputs
    (optionally as a captured CUDA graph), download() returns ScanResults, upload() re-copies the
    host inputs (end-to-end measurement)."""

    def __init__(self, ctx, scans, pipeline=None, seg_configs=None, rings=None, tuning=None):
        self.ctx = ctx
        self.pipeline = pipeline or PipelineConfig.default()
        n = len(scans)
        self._arrs = [_xyzi(s) for s in scans]
        self._rings = [None if (rings is None or rings[i] is None) else np.ascontiguousarray(rings[i], np.uint16)
                       for i in range(n)]
        cfgs = seg_configs or [SegmenterConfig.default() for _ in range(n)]
        self._ins = (ScanInput * n)()
        for i in range(n):
            self._ins[i] = ScanInput(self._arrs[i].ctypes.data,
                                     None if self._rings[i] is None else self._rings[i].ctypes.data,
                                     len(self._arrs[i]), cfgs[i])
        self._bufs = [ResultBuffers(len(a)) for a in self._arrs]
        h = ctypes.c_void_p()
        if tuning is None:
            check(library().lp_batch_create(ctx.handle, ctypes.byref(self.pipeline), self._ins, n, ctypes.byref(h)), ctx)
        else:
            check(library().lp_batch_create_tuned(ctx.handle, ctypes.byref(self.pipeline), self._ins, n,
                                                  ctypes.byref(tuning), ctypes.byref(h)), ctx)
        self.handle = h
        self.n = n

    @property
    def tuning(self):
        t = Tuning()
        check(library().lp_batch_get_tuning(self.handle, ctypes.byref(t)), self.ctx)
        return t

    @property
    def points(self):
        return int(library().lp_batch_points(self.handle))

    @property
    def device_bytes(self):
        return int(library().lp_batch_device_bytes(self.handle))

    def upload(self):
        check(library().lp_batch_upload(self.ctx.handle, self.handle), self.ctx)

    def execute(self):
        check(library().lp_batch_execute(self.ctx.handle, self.handle), self.ctx)

    def capture_graph(self):
        check(library().lp_batch_capture_graph(self.ctx.handle, self.handle), self.ctx)

    def synchronize(self):
        check(library().lp_context_synchronize(self.ctx.handle), self.ctx)

    def download(self):
        outs = (ScanOutput * self.n)(*[b.out for b in self._bufs])
        st = library().lp_batch_download(self.ctx.handle, self.handle, outs)
        for i in range(self.n):
            self._bufs[i].out = outs[i]
        check(st, self.ctx)
        return [b.result() for b in self._bufs]

    def time(self, iters, flush_l2=True):
        ms = ctypes.c_float()
        check(library().lp_batch_time(self.ctx.handle, self.handle, iters, 1 if flush_l2 else 0, ctypes.byref(ms)),
              self.ctx)
        return ms.value

    def profile(self, cap=256, name_len=48):
        names = ctypes.create_string_buffer(cap * name_len)
        ms = np.zeros(cap, np.float32)
        cnt = ctypes.c_uint32()
        check(library().lp_batch_profile(self.ctx.handle, self.handle, names, name_len, ptr(ms), cap,
                                         ctypes.byref(cnt)), self.ctx)
        k = min(cnt.value, cap)
        raw = names.raw
        return [(raw[i * name_len:(i + 1) * name_len].split(b"\0")[0].decode(), float(ms[i])) for i in range(k)]

    def close(self):
        if self.handle:
            library().lp_batch_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget_bytes", ctypes.c_uint64), ("max_batch_scans", ctypes.c_uint32),
                ("slots", ctypes.c_uint32)]


class ServerDone(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32), ("batch_scans", ctypes.c_uint32),
                ("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "failed", "batches", "scans_in_batches",
                                               "max_batch_seen", "pending", "device_bytes", "memory_waits")]


class Server:
    """Continuous-batching request loop (lp_server_*): submit scans as they arrive, poll results.
    Inputs and result buffers of a scan are kept alive here until it is polled."""

    def __init__(self, device=0, pipeline=None, memory_budget_bytes=20 << 30, max_batch_scans=16, slots=3):
        self.pipeline = pipeline or PipelineConfig.default()
        cfg = ServerConfig(memory_budget_bytes, max_batch_scans, slots)
        h = ctypes.c_void_p()
        check(library().lp_server_create(device, ctypes.byref(self.pipeline), ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._live = {}

    def submit(self, xyzi, ring, seg_config, tag):
        a = _xyzi(xyzi)
        r = None if ring is None else np.ascontiguousarray(ring, np.uint16)
        inp = ScanInput(a.ctypes.data, None if r is None else r.ctypes.data, len(a), seg_config)
        buf = ResultBuffers(len(a))
        self._live[int(tag)] = (a, r, inp, buf)
        check(library().lp_server_submit(self.handle, ctypes.byref(inp), ctypes.byref(buf.out), int(tag)))

    def poll(self, wait_us=1000, capacity=256):
        """[(ServerDone, ScanResult or None)] of scans finished since the last poll."""
        done = (ServerDone * capacity)()
        n = ctypes.c_uint32()
        check(library().lp_server_poll(self.handle, done, capacity, ctypes.byref(n), wait_us))
        out = []
        for i in range(n.value):
            d = done[i]
            _, _, _, buf = self._live.pop(int(d.tag))
            out.append((d, buf.result() if d.status == LP_OK else None))
        return out

    def hold(self, on=True):
        check(library().lp_server_hold(self.handle, 1 if on else 0))

    def stats(self):
        s = ServerStats()
        check(library().lp_server_stats_get(self.handle, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            library().lp_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchCall:
    """One lp_process_batch call with its argument arrays built once, for a caller that runs the
    same scan and result buffers call after call (page-locked buffers refilled in place, as a sensor
    node reuses its messages): run() is the C call alone, without rebuilding the per-scan structs.

    Binds the caller's arrays themselves, so they must need no conversion: scans float32, N x 4,
    C-contiguous; rings uint16, 1-D, C-contiguous (or None). Segmenter configs are copied here;
    the pipeline config is passed by reference on every run.
    """

    def __init__(self, scans, pipeline=None, seg_configs=None, rings=None, outputs=None):
        n = len(scans)
        for a in scans:
            if (not isinstance(a, np.ndarray) or a.dtype != np.float32 or a.ndim != 2 or a.shape[1] != 4
                    or not a.flags.c_contiguous):
                raise ValueError("BatchCall binds its scans: float32 N x 4 C-contiguous arrays")
        rr = [None if (rings is None or rings[i] is None) else rings[i] for i in range(n)]
        for r in rr:
            if r is not None and (not isinstance(r, np.ndarray) or r.dtype != np.uint16 or r.ndim != 1
                                  or not r.flags.c_contiguous):
                raise ValueError("BatchCall binds its rings: uint16 1-D C-contiguous arrays")
        cfgs = seg_configs or [SegmenterConfig.default() for _ in range(n)]
        bufs = list(outputs) if outputs is not None else []
        ins = (ScanInput * n)()
        for i in range(n):
            ins[i] = ScanInput(scans[i].ctypes.data, None if rr[i] is None else rr[i].ctypes.data, len(scans[i]),
                               cfgs[i])
            if outputs is None:
                bufs.append(ResultBuffers(len(scans[i])))
            elif len(bufs[i].seg) < len(scans[i]):
                raise ValueError("output buffers smaller than the scan")
        self.n = n
        self.pipeline = pipeline or PipelineConfig.default()
        self._keep = (list(scans), rr)  # the arrays ins points into
        self.ins = ins
        self.outs = (ScanOutput * n)(*[b.out for b in bufs])
        self.bufs = bufs

    def run(self, ctx, raw=True):
        st = library().lp_process_batch(ctx.handle, ctypes.byref(self.pipeline), self.ins, self.outs, self.n)
        for i in range(self.n):
            self.bufs[i].out = self.outs[i]
        check(st, ctx)
        return self.bufs if raw else [b.result() for b in self.bufs]


def process_batch(ctx, scans, pipeline=None, seg_configs=None, rings=None, outputs=None, raw=False):
    """Run the whole per-scan path on a batch of scans in one launch sequence.

    scans: list of N_i x 4 float32 arrays; seg_configs: list of SegmenterConfig (default each);
    rings: list of uint16 arrays or None. Returns a list of ScanResult. outputs: ResultBuffers to
    fill (reused across calls, e.g. pinned ones) instead of fresh buffers; raw=True returns those
    buffers (arrays filled in place, counts in .out) without building ScanResult objects.
    """
    arrs = [_xyzi(s) for s in scans]
    rr = None if rings is None else [None if r is None else np.ascontiguousarray(r, np.uint16).reshape(-1) for r in rings]
    return BatchCall(arrs, pipeline, seg_configs, rr, outputs).run(ctx, raw)
