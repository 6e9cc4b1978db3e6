"""Run-time tuning, host side (no GPU): the defaults and their ranges, a batch's bucket key, and the
tuning table's set / get / save / load through the C ABI."""
import numpy as np
import pytest

import lp_testlib as T

lp = T.lp


def seg(h, w):
    c = lp.SegmenterConfig.default()
    c.image_height = h
    c.image_width = w
    return c


def clouds(sizes):
    return [np.zeros((n, 4), np.float32) for n in sizes]


def test_defaults_and_ranges():
    t = lp.Tuning.default()
    assert t.as_dict() == {"parts": 0, "balance_parts": 0, "hull_cta_min": 512, "hull_ctas_per_sm": 2,
                           "cell_ctas_per_sm": 8, "jcp_ctas_per_sm": 8}
    assert t.valid()
    for field, good, bad in [("parts", [0, 1, 8], [9]), ("balance_parts", [0, 1], [2]),
                             ("hull_cta_min", [64, 512], [63, 513]), ("hull_ctas_per_sm", [1, 4], [0, 5]),
                             ("cell_ctas_per_sm", [1, 16], [0, 17]), ("jcp_ctas_per_sm", [1, 16], [0, 17])]:
        for v in good:
            assert lp.Tuning.default(**{field: v}).valid(), (field, v)
        for v in bad:
            assert not lp.Tuning.default(**{field: v}).valid(), (field, v)


def test_bucket_key():
    # scan-count classes
    for n, cls in [(1, 0), (2, 1), (15, 1), (16, 2), (31, 2), (32, 3), (63, 3), (64, 4), (100, 4)]:
        k = lp.tuning_key(clouds([10] * n), [seg(64, 2048)] * n)
        assert k.as_tuple() == (cls, 1, 1), n
    # ring / azimuth classes of the scans holding most points
    k = lp.tuning_key(clouds([100, 300, 50]), [seg(32, 1024), seg(128, 4096), seg(64, 2048)])
    assert k.as_tuple() == (1, 2, 2)
    k = lp.tuning_key(clouds([400, 300, 50]), [seg(32, 1024), seg(128, 4096), seg(64, 2048)])
    assert k.as_tuple() == (1, 0, 0)
    k = lp.tuning_key(clouds([100, 100]), [seg(33, 1025), seg(64, 2048)])
    assert k.as_tuple() == (1, 1, 1)  # boundaries: 33 rings and 1025 bins fall in the middle classes
    # a tie goes to the lower class
    k = lp.tuning_key(clouds([100, 100]), [seg(32, 1024), seg(128, 4096)])
    assert k.as_tuple() == (1, 0, 0)


def test_table_roundtrip(tmp_path):
    tab = lp.TuningTable()
    k1 = lp.TuningKey(4, 1, 2)
    k2 = lp.TuningKey(0, 2, 0)
    found, t, ms = tab.get(k1)
    assert not found and t.as_dict() == lp.Tuning.default().as_dict() and ms == 0.0
    a = lp.Tuning.default(parts=2, balance_parts=1, hull_cta_min=256, hull_ctas_per_sm=3, cell_ctas_per_sm=12,
                          jcp_ctas_per_sm=4)
    b = lp.Tuning.default(parts=8, hull_cta_min=128)
    tab.set(k1, a, 2.5)
    tab.set(k2, b, 0.75)
    assert len(tab) == 2
    found, t, ms = tab.get(k1)
    assert found and t.as_dict() == a.as_dict() and ms == pytest.approx(2.5)
    tab.set(k1, b, 1.0)  # replaces
    assert len(tab) == 2 and tab.get(k1)[1].as_dict() == b.as_dict()
    path = tmp_path / "tuning.txt"
    tab.save(path)
    text = path.read_text().splitlines()
    assert text[0].startswith("#") and len(text) == 3
    other = lp.TuningTable()
    other.set(lp.TuningKey(2, 0, 0), a, 9.0)
    other.load(path)  # adds and overrides
    assert len(other) == 3
    for k, want in [(k1, b), (k2, b), (lp.TuningKey(2, 0, 0), a)]:
        found, t, _ = other.get(k)
        assert found and t.as_dict() == want.as_dict()
    assert other.get(k2)[2] == pytest.approx(0.75)


def test_table_rejects_bad_entries(tmp_path):
    tab = lp.TuningTable()
    with pytest.raises(ValueError):
        tab.set(lp.TuningKey(5, 0, 0), lp.Tuning.default())  # no such scan-count class
    with pytest.raises(ValueError):
        tab.set(lp.TuningKey(0, 0, 0), lp.Tuning.default(hull_cta_min=1024))  # beyond the warp path's limit
    tab.set(lp.TuningKey(1, 1, 1), lp.Tuning.default(parts=2), 1.0)
    bad = tmp_path / "bad.txt"
    bad.write_text("# header\n1 1 1 2 0 512 2 8 8 1.0\n0 0 0 2 0 9999 2 8 8 1.0\n")
    with pytest.raises(ValueError):
        tab.load(bad)
    assert len(tab) == 1  # a malformed file changes nothing
    with pytest.raises(ValueError):
        tab.load(tmp_path / "missing.txt")
