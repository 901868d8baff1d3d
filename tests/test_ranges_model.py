"""RangesInt32 (intervals in numpy arrays) against a plain-list model of
the same semantics (include/Ranges.h:14-65, src/Ranges.cxx): random
sequences of appends without checks (unsorted, overlapping, empty, out of
range), add_interval, merges, complements, buffers, intersections and
slices give the same intervals and masks."""
import numpy as np
import pytest

from so3g_gb300.ranges import RangesInt32, RangesMatrix


class ListRanges:
    def __init__(self, count):
        self.count = count
        self.segs = []

    def cleanup(self):
        segs = sorted((max(0, a), min(self.count, b)) for a, b in self.segs)
        out = []
        for a, b in segs:
            if b <= a:
                continue
            if out and a <= out[-1][1]:
                out[-1][1] = max(out[-1][1], b)
            else:
                out.append([a, b])
        self.segs = out

    def complement(self):
        out, x = [], 0
        for a, b in sorted(self.segs):
            if a > x:
                out.append([x, a])
            x = max(x, b)
        if x < self.count:
            out.append([x, self.count])
        r = ListRanges(self.count)
        r.segs = out
        return r

    def mask(self):
        m = np.zeros(self.count, dtype=bool)
        for a, b in self.segs:
            m[max(a, 0):max(b, 0)] = True
        return m


def _random_pairs(rng, count, n):
    lo = rng.integers(-20, count + 20, n)
    return [[int(a), int(a + d)] for a, d in zip(lo, rng.integers(-5, 60, n))]


@pytest.mark.parametrize("seed", range(12))
def test_against_list_model(seed):
    rng = np.random.default_rng(seed)
    count = int(rng.integers(1, 400))
    r, m = RangesInt32(count), ListRanges(count)
    for a, b in _random_pairs(rng, count, int(rng.integers(0, 40))):
        r.append_interval_no_check(a, b)
        m.segs.append([a, b])
    assert r._segs == m.segs
    assert np.array_equal(r.mask(), m.mask())
    c, cm = r.complement(), m.complement()
    assert c._segs == cm.segs
    for a, b in _random_pairs(rng, count, 5):
        r.add_interval(a, b)
        m.segs.append([a, b])
        m.cleanup()
        assert r._segs == m.segs
    o = RangesInt32(count)
    om = ListRanges(count)
    for a, b in _random_pairs(rng, count, 10):
        o.append_interval_no_check(a, b)
        om.segs.append([a, b])
    both = r.copy().merge(o)
    mm = ListRanges(count)
    mm.segs = [list(s) for s in m.segs] + [list(s) for s in om.segs]
    mm.cleanup()
    assert both._segs == mm.segs
    buf = r.buffered(3)
    bm = ListRanges(count)
    bm.segs = [[a - 3, b + 3] for a, b in m.segs]
    bm.cleanup()
    assert buf._segs == bm.segs
    lo, hi = sorted(int(x) for x in rng.integers(0, count + 1, 2))
    sl = r[lo:hi]
    want = [[max(a, lo) - lo, min(b, hi) - lo] for a, b in m.segs if min(b, hi) > max(a, lo)]
    assert sl._segs == want and sl.count == hi - lo and sl.reference == lo
    o.add_interval(0, 0)   # fold and normalise
    om.cleanup()
    inter = r * o
    cover = m.mask() & om.mask()
    assert np.array_equal(inter.mask(), cover)
    assert np.array_equal(r.ranges(), np.array(m.segs, dtype=np.int32).reshape(-1, 2))


def test_from_mask_and_array_roundtrip():
    rng = np.random.default_rng(3)
    mask = rng.random((7, 1000)) < 0.3
    rm = RangesMatrix.from_mask(mask)
    assert np.array_equal(rm.mask(), mask)
    for row, r in zip(mask, rm):
        again = RangesInt32.from_array(r.ranges(), len(row))
        assert np.array_equal(again.mask(), row)
    assert RangesInt32.from_mask(np.zeros(0, dtype=bool))._segs == []
    assert RangesInt32(5).complement()._segs == [[0, 5]]
    assert RangesInt32(0).complement()._segs == []
