"""lp_convex_hull_noalloc: the hull entry point for callers that cannot allocate device memory
(its working memory is a static device array inside the library). Checked through the C ABI
against the oracle's convexHull and against lp_convex_hull on two calls in a row, a large then a
small polygon, so that leftovers of the first call in the shared array would show. The caller's
buffers are device tensors."""
import ctypes

import numpy as np
import pytest

import lp_testlib as T

lp = T.lp
pytestmark = pytest.mark.gpu


def _noalloc():
    f = lp.library().lp_convex_hull_noalloc
    f.restype = ctypes.c_int32
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return f


def test_noalloc_hull_matches_lp_convex_hull(ctx):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for torch")
    fn = _noalloc()
    poly = lp.Polygonizer(ctx)
    rng = np.random.default_rng(2024)
    for n in (40000, 700):  # two calls in a row: the second reuses the array the first filled
        pts = (rng.normal(size=(n, 2)) * 8.0).astype(np.float32).astype(np.float64)
        pts[: n // 10] = np.round(pts[: n // 10], 1)  # duplicates and collinear runs
        want = T.o_hull(pts)
        assert np.array_equal(poly.convexHull(pts), want)
        d_xy = torch.from_numpy(pts).cuda()
        d_out = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
        d_n = torch.zeros(1, dtype=torch.int32, device="cuda")
        st = fn(d_xy.data_ptr(), n, d_out.data_ptr(), d_n.data_ptr(), None)
        assert st == lp.LP_OK
        torch.cuda.synchronize()
        h = int(d_n.item())
        got = d_out[:h].cpu().numpy()
        assert h == len(want)
        assert np.array_equal(got, want)


def test_noalloc_hull_small_and_capacity(ctx):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device for torch")
    fn = _noalloc()
    d_xy = torch.tensor([[3.0, 1.0], [1.0, 2.0]], dtype=torch.float64, device="cuda")
    d_out = torch.full((4,), -7, dtype=torch.int32, device="cuda")
    d_n = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert fn(d_xy.data_ptr(), 2, d_out.data_ptr(), d_n.data_ptr(), None) == lp.LP_OK
    torch.cuda.synchronize()
    assert int(d_n.item()) == 2 and d_out[:2].cpu().tolist() == [0, 1]  # reference: iota below 3 points
    too_many = 65536 + 1
    assert fn(d_xy.data_ptr(), too_many, d_out.data_ptr(), d_n.data_ptr(), None) == lp.LP_ERR_CAPACITY
