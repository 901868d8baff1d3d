"""Projection parity on the GPU: to_map, to_weight_map and from_map of the
CUDA library against the CPU oracle on the same seeded inputs.

Every pointing mode is checked, for every coordinate system.  CEA's
longitude comes from the math library's atan2 (src/Projection.cxx:468),
whose CUDA and host roundings may differ in the last bit; that moves a
pixel index only for a sample within ~1e-16 of a pixel edge, which these
inputs do not have, so CEA is held to the same bounds.  Tolerances: from_map evaluates each
sample exactly as the reference does and is compared bit for bit.
to_map/to_weight_map form every float32 term exactly as the reference does;
only the order of the float64 sums differs (atomics, and the warp
pre-reduction of pixel runs), so they must agree to 1e-12 of the map's
scale.  The one exception is the certified pointing of bilinear maps,
whose interpolation weights are within one float32 ulp of the reference's:
there maps and signals agree to 1e-6 of their scale.
"""
import numpy as np
import pytest

import so3g_gb300
from so3g_gb300 import _abi
from conftest import bits_equal
from helpers import Case, oracle_map, map_from_oracle, stack_map

pytestmark = pytest.mark.gpu

RTOL = 1e-12
RTOL_BILINEAR_CERTIFIED = 1e-6
ACCUMS = [_abi.ACCUM_ATOMIC, _abi.ACCUM_WARP_RUNS]
RTOL_MIXED = 1e-6
MODES = [_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED, _abi.POINTING_MIXED]


def rtol_for(bil, mode, coord="CAR"):
    """Map/signal tolerance against the float64 oracle: mixed pointing on
    CAR, TAN, ZEA, SIN and ARC maps evaluates spin factors, bilinear weights
    and from_map terms in float32; certified bilinear weights are within one
    float32 ulp; every other case forms each float32 term as the reference
    does."""
    if mode == _abi.POINTING_MIXED and coord in ("CAR", "TAN", "ZEA", "SIN", "ARC") and not bil:
        return RTOL_MIXED
    if bil and mode != _abi.POINTING_EXACT:
        return RTOL_BILINEAR_CERTIFIED
    return RTOL


def close(got, want, rtol=RTOL):
    got, want = stack_map(got), stack_map(want)
    scale = max(np.abs(want).max(), 1e-300)
    err = np.abs(got - want).max()
    assert err <= rtol * scale, (err, scale)


def oracle_to_map(orc, c, m, det_weights=None, threads=None):
    flat, offs = oracle_map(m)
    err = orc.to_map(c.pz, c.bore, c.dets, c.resp, c.signal, det_weights, flat, offs, threads)
    return map_from_oracle(flat, offs, m), err


def oracle_to_weight(orc, c, m, det_weights=None, threads=None):
    flat, offs = oracle_map(m)
    err = orc.to_weight_map(c.pz, c.bore, c.dets, c.resp, det_weights, flat, offs, threads)
    return map_from_oracle(flat, offs, m), err


CASES = [(coord, tiled, bil)
         for coord in ["CAR", "CEA", "TAN", "ZEA", "ARC", "SIN", "Flat", "Quat"]
         for tiled in (False, True) for bil in (False, True)]


@pytest.mark.parametrize("coord,tiled,bil", CASES)
@pytest.mark.parametrize("ncomp", [1, 3])
@pytest.mark.parametrize("mode", MODES)
def test_to_map(orc, gpulib, coord, tiled, bil, ncomp, mode):
    c = Case(orc, coord=coord, ncomp=ncomp, tiled=tiled, bilinear=bil, n_det=5, n_time=4000)
    c.eng.pointing = mode
    want, _ = oracle_to_map(orc, c, c.blank((ncomp,)))
    for accum in ACCUMS:
        got = c.eng.to_map(c.blank((ncomp,)), c.bore, c.dets, c.resp, c.signal, None, None,
                           accum=accum)
        close(got, want, rtol_for(bil, mode, coord))


@pytest.mark.parametrize("coord,tiled,bil", CASES)
@pytest.mark.parametrize("ncomp", [2, 3])
@pytest.mark.parametrize("mode", MODES)
def test_to_weight_map(orc, gpulib, coord, tiled, bil, ncomp, mode):
    c = Case(orc, coord=coord, ncomp=ncomp, tiled=tiled, bilinear=bil, n_det=5, n_time=4000)
    c.eng.pointing = mode
    want, _ = oracle_to_weight(orc, c, c.blank((ncomp, ncomp)))
    for accum in ACCUMS:
        got = c.eng.to_weight_map(c.blank((ncomp, ncomp)), c.bore, c.dets, c.resp, None, None,
                                  accum=accum)
        close(got, want, rtol_for(bil, mode, coord))


@pytest.mark.parametrize("coord,tiled,bil", CASES)
@pytest.mark.parametrize("ncomp", [1, 2, 3])
@pytest.mark.parametrize("mode", MODES)
def test_from_map(orc, gpulib, coord, tiled, bil, ncomp, mode):
    c = Case(orc, coord=coord, ncomp=ncomp, tiled=tiled, bilinear=bil, n_det=5, n_time=4000)
    c.eng.pointing = mode
    m = c.random_map((ncomp,))
    sig0 = np.random.default_rng(3).standard_normal((5, 4000)).astype(np.float32)
    want = sig0.copy()
    flat, offs = oracle_map(m)
    orc.from_map(c.pz, c.bore, c.dets, c.resp, flat, want, offs)
    got = sig0.copy()
    ret = c.eng.from_map(m, c.bore, c.dets, c.resp, got)
    tol = rtol_for(bil, mode, coord)
    exact = tol == RTOL
    if exact:
        assert bits_equal(got, want)
    else:
        close(got, want, tol)
    assert all(np.shares_memory(r, got) for r in ret)
    # signal=None creates zeros.
    fresh = np.array(c.eng.from_map(m, c.bore, c.dets, c.resp, None))
    want0 = np.zeros_like(sig0)
    orc.from_map(c.pz, c.bore, c.dets, c.resp, flat, want0, offs)
    if exact:
        assert bits_equal(fresh, want0)
    else:
        close(fresh, want0, tol)


def test_map_accumulates_and_returns_same_object(orc, gpulib):
    c = Case(orc, coord="CAR", n_det=4, n_time=3000)
    m = c.random_map((3,))
    m0 = m.copy()
    ret = c.eng.to_map(m, c.bore, c.dets, c.resp, c.signal, None, None)
    assert ret is m
    want, _ = oracle_to_map(orc, c, m0.copy())
    close(m, want)


def test_det_weights(orc, gpulib):
    c = Case(orc, coord="CAR", n_det=4, n_time=3000)
    w = np.array([0., 2., 0.5, 0.], dtype=np.float32)
    got = c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, w, None)
    want, _ = oracle_to_map(orc, c, c.blank((3,)), det_weights=w)
    close(got, want)
    gw = c.eng.to_weight_map(None, c.bore, c.dets, c.resp, w, None)
    ww, _ = oracle_to_weight(orc, c, c.blank((3, 3)), det_weights=w)
    close(gw, ww)
    # All-zero weights: nothing projected (test/test_proj_eng.py:71-74).
    z = c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal,
                     np.zeros(4, np.float32), None)
    assert np.all(z == 0)


def test_thread_intervals(orc, gpulib):
    """Every form of thread_intervals, including overlapping ranges (which
    the reference projects twice)."""
    from so3g_gb300 import RangesInt32, RangesMatrix
    c = Case(orc, coord="CAR", n_det=3, n_time=3000)
    rng = np.random.default_rng(4)

    def rm():
        rows = []
        for d in range(3):
            r = RangesInt32(3000)
            for _ in range(4):
                a = int(rng.integers(0, 2900))
                r.append_interval_no_check(a, min(3000, a + int(rng.integers(1, 400))))
            rows.append(r)
        return RangesMatrix(rows)

    forms = [rm(), RangesMatrix([rm(), rm()]), [RangesMatrix([rm(), rm()]), RangesMatrix([rm()])]]
    # These thread lists are not pixel-disjoint, so the oracle must not run
    # its threads concurrently (the reference would race the same way).
    orc.set_threads(1)
    for th in forms:
        got = c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, None, th)
        want, _ = oracle_to_map(orc, c, c.blank((3,)), threads=th)
        close(got, want)
        gw = c.eng.to_weight_map(None, c.bore, c.dets, c.resp, None, th)
        ww, _ = oracle_to_weight(orc, c, c.blank((3, 3)), threads=th)
        close(gw, ww)
    import os
    orc.set_threads(os.cpu_count() or 1)


def test_thread_intervals_shape_errors(orc, gpulib):
    from so3g_gb300 import RangesInt32, RangesMatrix
    c = Case(orc, coord="CAR", n_det=3, n_time=300)
    bad_det = RangesMatrix([RangesInt32(300) for _ in range(2)])
    with pytest.raises(RuntimeError, match="n_det=3"):
        c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, None, bad_det)
    bad_time = RangesMatrix([RangesInt32(299) for _ in range(3)])
    with pytest.raises(RuntimeError, match="n_time=300"):
        c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, None, bad_time)


@pytest.mark.parametrize("mode", MODES)
def test_missing_tile_raises(orc, gpulib, mode):
    c = Case(orc, coord="CAR", tiled=True, n_det=4, n_time=3000)
    c.eng.pointing = mode
    hits = np.array(c.eng.tile_hits(c.bore, c.dets))
    hit = np.nonzero(hits)[0]
    assert len(hit) > 1
    # Leave out one hit tile: projecting onto it is an error
    # (src/Projection.cxx:1084-1088).
    pop = [t for t in c.all_tiles() if t != hit[0]]
    m = c.blank((3,), populate=pop)
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index %d\)" % hit[0]):
        c.eng.to_map(m, c.bore, c.dets, c.resp, c.signal, None, None)
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index %d\)" % hit[0]):
        c.eng.from_map(c.random_map((3,), populate=pop), c.bore, c.dets, c.resp, None)


def test_active_tiles_zeros(orc, gpulib):
    c = Case(orc, coord="CAR", tiled=True, n_det=4, n_time=3000, active=[0, 3])
    z = c.eng.zeros(3)
    assert [i for i, t in enumerate(z) if t is not None] == [0, 3]
    z[0] = None
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index 0\): Projector expects"):
        c.eng.to_map(z, c.bore, c.dets, c.resp, c.signal, None, None)


def test_tiled_equals_untiled(orc, gpulib):
    """Tiled maps hold the untiled map's pixels (demos/demo_proj1.py
    invariant), within the float64 summation-order tolerance -- except row
    and column 0: the Tiled nearest-neighbour pixelizor truncates x in
    (-1, 0) to column 0 (src/Projection.cxx:1126-1129) where NonTiled
    rejects it (:917-918), so samples just off the map's low edges land
    there only in the tiled map."""
    c = Case(orc, coord="CAR", tiled=True, n_det=5, n_time=4000)
    u = Case(orc, coord="CAR", tiled=False, n_det=5, n_time=4000)
    mt = c.eng.to_map(c.blank((3,)), c.bore, c.dets, c.resp, c.signal, None, None)
    mu = u.eng.to_map(None, u.bore, u.dets, u.resp, u.signal, None, None)
    ty, tx = c.eng.tile_shape
    ntx = c.eng.tile_grid[1]
    re = np.zeros_like(mu)
    for i, t in enumerate(mt):
        r, q = divmod(i, ntx)
        re[:, r * ty:r * ty + t.shape[1], q * tx:q * tx + t.shape[2]] = t
    close(re[:, 1:, 1:], mu[:, 1:, 1:])
    # The edge difference is the oracle's too.
    want, _ = oracle_to_map(orc, c, c.blank((3,)))
    close(mt, want)


def test_device_mode(orc, gpulib):
    import torch
    c = Case(orc, coord="CAR", n_det=4, n_time=3000)
    b, d = torch.from_numpy(c.bore).cuda(), torch.from_numpy(c.dets).cuda()
    r, s = torch.from_numpy(c.resp).cuda(), torch.from_numpy(c.signal).cuda()
    m = c.eng.to_map(None, b, d, r, s, None, None)
    assert isinstance(m, torch.Tensor) and m.is_cuda
    want, _ = oracle_to_map(orc, c, c.blank((3,)))
    close(m.cpu().numpy(), want)
    # In place into a strided signal view (row stride != n_time).
    big = torch.zeros((4, 3500), dtype=torch.float32, device="cuda")
    view = big[:, 100:3100]
    c.eng.from_map(m, b, d, r, view)
    w = np.zeros((4, 3000), np.float32)
    orc.from_map(c.pz, c.bore, c.dets, c.resp, m.cpu().numpy().ravel().copy(), w)
    assert bits_equal(view.cpu().numpy(), w)
    assert float(big[:, :100].abs().sum()) == 0.0


def test_errors_match_reference(orc, gpulib):
    c = Case(orc, coord="CAR", n_det=2, n_time=100)
    with pytest.raises(RuntimeError, match="has incompatible shape"):
        c.eng.to_map(np.zeros((1,) + c.eng._pix_shape()), c.bore, c.dets, c.resp, c.signal,
                     None, None)
    dets = c.dets.copy()
    dets[1, 0] = np.nan
    with pytest.raises(ValueError, match="nan found at index 1"):
        c.eng.to_map(None, c.bore, dets, c.resp, c.signal, None, None)
    with pytest.raises(ValueError, match="nan found at index 1"):
        c.eng.to_weight_map(None, c.bore, dets, c.resp, None, None)
    with pytest.raises(ValueError, match="float32"):
        c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal.astype(np.float64), None, None)
    with pytest.raises(TypeError, match="buffer protocol"):
        c.eng.to_map(None, "boresight", c.dets, c.resp, c.signal, None, None)
