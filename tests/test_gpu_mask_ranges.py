"""Cut masks to sample ranges on the device: RangesMatrix.from_mask of a
CUDA mask (python/proj/ranges.py:11-297) against the host RangesMatrix of
the same mask, segment for segment, and projections that take either as
thread_intervals."""
import numpy as np
import pytest

from so3g_gb300 import synth
from so3g_gb300.projeng import flatten_ranges
from so3g_gb300.ranges import DeviceRangesMatrix, RangesMatrix

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60


def random_mask(n_det, n_time, seed):
    """Runs of random length, rows all set / all clear, runs touching both
    ends of the row and single-sample runs."""
    rng = np.random.default_rng(seed)
    m = np.zeros((n_det, n_time), bool)
    for d in range(n_det):
        kind = d % 5
        if kind == 0:
            m[d] = True
        elif kind == 1:
            continue
        elif kind == 2:
            m[d] = rng.random(n_time) < 0.5         # many short runs
        else:
            t = 0
            on = bool(d % 2)
            while t < n_time:
                L = int(rng.integers(1, 200 if kind == 3 else 5000))
                m[d, t:t + L] = on
                on = not on
                t += L
    return m


def host_segments(m):
    seg, _, _ = flatten_ranges([[RangesMatrix.from_mask(m)]])
    return seg


@pytest.mark.parametrize("n_time", [1, 15, 16, 17, 4096, 4113, 100_003])
def test_segments_match_host(gpulib, n_time):
    import torch
    m = random_mask(23, n_time, n_time)
    dr = RangesMatrix.from_mask(torch.from_numpy(m).cuda())
    assert isinstance(dr, DeviceRangesMatrix)
    assert dr.shape == m.shape
    want = host_segments(m)
    got = dr.seg.cpu().numpy()
    assert np.array_equal(got, want)
    lens = want[:, 2] - want[:, 1]
    assert dr.max_len == (int(lens.max()) if len(lens) else 0)
    assert np.array_equal(dr.mask(), m)


def test_unaligned_rows_and_uint8(gpulib):
    """Rows that do not start on 16-byte boundaries (a column slice) and a
    uint8 mask with values other than 0 and 1."""
    import torch
    m = random_mask(9, 5000, 7)
    big = np.zeros((9, 5003), np.uint8)
    big[:, 3:] = m * np.uint8(200)
    t = torch.from_numpy(big).cuda()[:, 3:]
    dr = RangesMatrix.from_mask(t)
    assert np.array_equal(dr.seg.cpu().numpy(), host_segments(m))


def test_projection_with_device_ranges(gpulib):
    import torch
    Q, dets, resp, gamma, sig = synth.workload(40, 60_000, seed=4, radius_deg=1.0)
    p = synth.car_projectionist((400, 500), 1 * ARCMIN)
    eng = p.get_ProjEng("TQU")
    q = synth.native(p, Q)
    m = random_mask(40, 60_000, 3)
    qd, dd, rd, sd = (torch.from_numpy(np.ascontiguousarray(x)).cuda()
                      for x in (q, dets, resp, sig))
    host_r = RangesMatrix.from_mask(m)
    dev_r = RangesMatrix.from_mask(torch.from_numpy(m).cuda())
    a = eng.to_map(None, qd, dd, rd, sd, None, host_r).cpu().numpy()
    b = eng.to_map(None, qd, dd, rd, sd, None, dev_r).cpu().numpy()
    scale = np.abs(a).max()
    assert scale > 0
    assert np.abs(a - b).max() <= 1e-12 * scale
    wa = eng.to_weight_map(None, qd, dd, rd, None, host_r).cpu().numpy()
    wb = eng.to_weight_map(None, qd, dd, rd, None, dev_r).cpu().numpy()
    assert np.abs(wa - wb).max() <= 1e-12 * np.abs(wa).max()
    # Host signal, device ranges: the signal goes through the device whole.
    c = eng.to_map(None, qd, dd, rd, sig, None, dev_r).cpu().numpy()
    assert np.abs(a - c).max() <= 1e-12 * scale


def test_device_ranges_shape_checked(gpulib):
    import torch
    Q, dets, resp, gamma, sig = synth.workload(4, 1000, seed=1)
    p = synth.car_projectionist((100, 100), 1 * ARCMIN)
    eng = p.get_ProjEng("T")
    q = synth.native(p, Q)
    dr = RangesMatrix.from_mask(torch.ones((5, 1000), dtype=torch.bool, device="cuda"))
    with pytest.raises(RuntimeError, match="n_det=4 but encountered n_det=5"):
        eng.to_map(None, q, dets, resp, sig, None, dr)
    dr = RangesMatrix.from_mask(torch.ones((4, 999), dtype=torch.bool, device="cuda"))
    with pytest.raises(RuntimeError, match="n_time=1000 but encountered n_time=999"):
        eng.to_map(None, q, dets, resp, sig, None, dr)
    empty = RangesMatrix.from_mask(torch.zeros((4, 1000), dtype=torch.bool, device="cuda"))
    assert empty.n_seg == 0 and empty.max_len == 0
    out = eng.to_map(None, q, dets, resp, sig, None, empty)
    assert not np.asarray(out).any()
