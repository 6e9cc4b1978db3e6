"""The C-ABI library loads without a GPU and exports every entry point declared in include/*.h."""
import ctypes
import os
import re

import numpy as np

import lp_testlib as T

INCLUDE = os.path.join(T.REPO, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**(lp_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def test_headers_declare_the_reference_replacements():
    names = declared_functions()
    for fn in ["lp_add_ring_info", "lp_segment", "lp_noise_remove", "lp_cluster", "lp_convex_hull",
               "lp_antipodal_pairs", "lp_bounding_box_rotating_calipers", "lp_bounding_box_pca",
               "lp_process_scan", "lp_process_batch", "lp_batch_create", "lp_batch_execute"]:
        assert fn in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(T.lp.LIB_PATH)
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_context_without_device_reports_status(built):
    lib = T.lp.library()
    h = ctypes.c_void_p()
    st = lib.lp_context_create(0, ctypes.byref(h))
    # on a machine without a GPU the library reports it instead of falling back to the CPU
    assert st in (T.lp.LP_OK, T.lp.LP_ERR_NO_DEVICE, T.lp.LP_ERR_CUDA)
    if st == T.lp.LP_OK:
        lib.lp_context_destroy(h)
    assert lib.lp_status_string(T.lp.LP_ERR_CAPACITY) == b"capacity exceeded"


def test_config_defaults_match_reference_structs(built):
    lib = T.lp.library()
    for name, cls in [("lp_segmenter_config_default", T.lp.SegmenterConfig),
                      ("lp_noise_remover_config_default", T.lp.NoiseRemoverConfig),
                      ("lp_clusterer_config_default", T.lp.ClustererConfig)]:
        c = cls()
        getattr(lib, name)(ctypes.byref(c))
        d = cls.default()
        for f, _ in cls._fields_:
            assert np.float32(getattr(c, f)) == np.float32(getattr(d, f)), (name, f)


def test_xyzrgb_record_matches_the_c_struct():
    """lp_xyzrgb (x, y, z float32; r, g, b, a uint8) is 16 bytes; the Python dtype mirrors it."""
    dt = T.lp.XYZRGB
    assert dt.itemsize == 16
    assert [dt.fields[f][1] for f in ("x", "y", "z", "r", "g", "b", "a")] == [0, 4, 8, 12, 13, 14, 15]


def test_bench_reads_traffic_ratios_from_profiles():
    """bench.py's roofline traffic comes from the `traffic_ratio <kernel> <ratio>` line of the ncu
    summaries under profiles/ (one per dominant kernel it may report)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(T.REPO, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    for kernel in ("k_hull", "k_jcp_rows"):
        t = bench.traffic_bytes(kernel, 1_000_000)
        assert t is not None and 0 < t < 10_000_000, (kernel, t)
    assert bench.traffic_bytes("no_such_kernel", 1_000_000) is None
