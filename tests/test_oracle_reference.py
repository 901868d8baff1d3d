"""The oracle against the reference itself: so3g's own ProjectionEngine,
compiled here from its src/Projection.cxx (oracle/ref_engine.cpp with the
stand-in headers of oracle/refstub), on the same seeded inputs.

Every coordinate system, spin, tiling and interpolation, and HEALPix:
coords, pixels, pointing_matrix, from_map, to_map and to_weight_map (both
single-threaded: the same summation order, so bit for bit), tile_hits and
pixel_ranges; the Precomp engines; and the reference's exception classes
and messages for bad inputs, against this library's ProjEng classes.

The one piece not pinned: boost's quaternion product (boost is absent;
the stand-in and the oracle both sum each component left to right).
These tests run where the reference checkout is (the CPU suite); the GPU
tests compare the CUDA library with the oracle."""
import numpy as np
import pytest

from conftest import bits_equal
from helpers import COORDS, Case, oracle_map, stack_map

ref_engine = pytest.importorskip("oracle.ref_engine")
if not ref_engine.available():
    pytest.skip("the so3g reference checkout is not available", allow_module_level=True)

N_DET, N_TIME = 4, 1500
FLAT = [(coord, ncomp, tiled, bil) for coord in COORDS for ncomp in (1, 2, 3)
        for tiled in (False, True) for bil in (False, True)]


def _ref(c):
    return ref_engine.RefEngine(c.name, c.args)


def _check_pointing(orc, c, r):
    assert bits_equal(np.asarray(r.coords(c.bore, c.dets, None)),
                      orc.coords(c.pz, c.bore, c.dets))
    ic = c.eng.index_count
    assert r.index_count == ic and r.comp_count == c.ncomp
    assert np.array_equal(np.asarray(r.pixels(c.bore, c.dets, None)),
                          orc.pixels(c.pz, c.bore, c.dets, ic))
    pix, proj = r.pointing_matrix(c.bore, c.dets, c.resp, None, None)
    wpix, wproj = orc.pointing_matrix(c.pz, c.bore, c.dets, c.resp, ic)
    assert np.array_equal(np.asarray(pix), wpix)
    assert bits_equal(np.asarray(proj), wproj)


def _check_maps(orc, c, r):
    nc = c.ncomp
    # to_map / to_weight_map into blank maps (every tile present).
    got = r.to_map(c.blank((nc,)), c.bore, c.dets, c.resp, c.signal, None, None)
    flat, offs = oracle_map(c.blank((nc,)))
    orc.to_map(c.pz, c.bore, c.dets, c.resp, c.signal, None, flat, offs)
    assert bits_equal(stack_map(got), flat)
    gw = r.to_weight_map(c.blank((nc, nc)), c.bore, c.dets, c.resp, None, None)
    wf, wo = oracle_map(c.blank((nc, nc)))
    orc.to_weight_map(c.pz, c.bore, c.dets, c.resp, None, wf, wo)
    assert bits_equal(stack_map(gw), wf)
    # det_weights: zero skips a detector, others scale its terms.
    dw = np.array([1., 0., 0.5, 2.], np.float32)
    got = r.to_map(c.blank((nc,)), c.bore, c.dets, c.resp, c.signal, dw, None)
    flat, offs = oracle_map(c.blank((nc,)))
    orc.to_map(c.pz, c.bore, c.dets, c.resp, c.signal, dw, flat, offs)
    assert bits_equal(stack_map(got), flat)
    # from_map of a random map, into zeros and into a given signal.
    m = c.random_map((nc,))
    sf, so = oracle_map(m)
    for base in (None, np.random.default_rng(3).standard_normal((N_DET, N_TIME),
                                                                dtype=np.float32)):
        want = np.zeros((N_DET, N_TIME), np.float32) if base is None else base.copy()
        orc.from_map(c.pz, c.bore, c.dets, c.resp, sf, want, so)
        got = np.asarray(r.from_map(m, c.bore, c.dets, c.resp,
                                    None if base is None else base.copy()))
        assert bits_equal(got, want)


def _labels(ranges, n_domain):
    """pixel_ranges output -> per-sample domain labels (the serial bunch:
    n_domain; unassigned: -1)."""
    lab = np.full((N_DET, N_TIME), -1, np.int32)
    for bunch, base in zip(ranges, (0, n_domain)):
        for k, dom in enumerate(bunch):
            for det, (count, segs) in enumerate(dom):
                assert count == N_TIME
                for a, b in segs:
                    lab[det, a:b] = base + k
    return lab


@pytest.mark.parametrize("coord,ncomp,tiled,bil", FLAT)
def test_flat_engines(orc, coord, ncomp, tiled, bil):
    c = Case(orc, coord=coord, ncomp=ncomp, tiled=tiled, bilinear=bil, n_det=N_DET,
             n_time=N_TIME, seed=31)
    r = _ref(c)
    _check_pointing(orc, c, r)
    _check_maps(orc, c, r)
    if tiled:
        hits = np.asarray(r.tile_hits(c.bore, c.dets))
        assert np.array_equal(hits, orc.tile_hits(c.pz, c.bore, c.dets, c.eng._n_tile()))
    if ncomp == 1 and not tiled:
        lab = _labels(r.pixel_ranges(c.bore, c.dets, None, 3), 3)
        assert np.array_equal(lab, orc.labels(c.pz, c.bore, c.dets, 0, 3))


@pytest.mark.parametrize("nside,nest,tiled", [(64, False, False), (64, True, False),
                                              (1024, False, False), (64, True, True)])
@pytest.mark.parametrize("ncomp", [1, 3])
def test_healpix_engines(orc, nside, nest, tiled, ncomp):
    c = Case(orc, coord="CAR", ncomp=ncomp, tiled=tiled, hp=(nside, nest, 4 if tiled else None),
             n_det=N_DET, n_time=N_TIME, seed=33)
    r = _ref(c)
    _check_pointing(orc, c, r)
    _check_maps(orc, c, r)
    if tiled:
        hits = np.asarray(r.tile_hits(c.bore, c.dets))
        assert np.array_equal(hits, orc.tile_hits(c.pz, c.bore, c.dets, c.eng._n_tile()))


def test_precomp_engines(orc):
    c = Case(orc, coord="CAR", ncomp=3, n_det=N_DET, n_time=N_TIME, seed=35)
    r = _ref(c)
    pix, proj = (np.asarray(x) for x in r.pointing_matrix(c.bore, c.dets, c.resp, None, None))
    pc = ref_engine.RefEngine("ProjEng_Precomp_NonTiled")
    naxis = c.eng.naxis
    m = pc.to_map(np.zeros((3,) + tuple(naxis)), pix, proj, c.signal, None, None)
    want = np.zeros(3 * naxis[0] * naxis[1])
    orc.precomp_to_map(pix, proj, c.signal, None, want, naxis=naxis)
    assert bits_equal(np.asarray(m).ravel(), want)
    w = pc.to_weight_map(np.zeros((3, 3) + tuple(naxis)), pix, proj, None, None)
    wwant = np.zeros(9 * naxis[0] * naxis[1])
    orc.precomp_to_weight_map(pix, proj, None, wwant, naxis=naxis)
    assert bits_equal(np.asarray(w).ravel(), wwant)
    src = np.random.default_rng(5).standard_normal((3,) + tuple(naxis))
    got = np.asarray(pc.from_map(src, pix, proj, None))
    swant = np.zeros((N_DET, N_TIME), np.float32)
    orc.precomp_from_map(pix, proj, src.ravel().copy(), swant, naxis=naxis)
    assert bits_equal(got, swant)


def _raises_same(call_ref, call_ours):
    with pytest.raises(Exception) as want:
        call_ref()
    with pytest.raises(Exception) as got:
        call_ours()
    assert type(got.value) is type(want.value), (got.value, want.value)
    assert str(got.value) == str(want.value)


def test_error_classes_and_messages(orc):
    """The library's ProjEng raises the reference's exception class with
    the reference's message for the binding's error cases."""
    c = Case(orc, coord="CAR", ncomp=3, n_det=N_DET, n_time=N_TIME, seed=37)
    r, e = _ref(c), c.eng
    bad_dets = c.dets.copy()
    bad_dets[2, 1] = np.nan
    cases = [
        ("nan detector", lambda x: x.coords(c.bore, bad_dets, None)),
        ("float32 boresight", lambda x: x.coords(c.bore.astype(np.float32), c.dets, None)),
        ("boresight shape", lambda x: x.pixels(c.bore[:, :3], c.dets, None)),
        ("signal dtype", lambda x: x.to_map(None, c.bore, c.dets, c.resp,
                                            c.signal.astype(np.float64), None, None)),
        ("signal rows", lambda x: x.to_map(None, c.bore, c.dets, c.resp, c.signal[:2], None,
                                           None)),
        # (A map of the right component count but other pixel axes is not
        # checked by the reference, which then writes out of bounds; this
        # library raises there, tests/test_host_api.py.)
        ("map components", lambda x: x.to_map(np.zeros((2,) + tuple(e.naxis)), c.bore, c.dets,
                                              c.resp, c.signal, None, None)),
        ("weight map components", lambda x: x.to_weight_map(
            np.zeros((3, 2) + tuple(e.naxis)), c.bore, c.dets, c.resp, None, None)),
        ("response shape", lambda x: x.from_map(np.zeros((3,) + tuple(e.naxis)), c.bore,
                                                c.dets, c.resp[:, :1], None)),
        ("not a buffer", lambda x: x.coords("boresight", c.dets, None)),
    ]
    for what, f in cases:
        _raises_same(lambda: f(r), lambda: f(e))
    # (A sample on a missing tile: the reference throws inside an OpenMP
    # region, which ends the process; the library raises the reference's
    # RuntimeError "Tiling problem (index i): ..." instead -- GPU tests.)
    # An nside that is not a power of two.
    _raises_same(lambda: ref_engine.RefEngine("ProjEng_HP_T_NonTiled", (100, 1, None, None)),
                 lambda: type(Case(orc, hp=(64, 1, None), ncomp=1).eng)((100, 1, None, None)))
