"""HEALPix parity on the GPU (ProjEng_HP_*): pixel indices, to_map,
to_weight_map and from_map against the oracle, plus the reference demo's
invariant that Tiled (NEST) maps are the untiled NEST map cut into tiles.

Pixel indices depend on cos/sin of the colatitude; CUDA's and the host
libm's may differ in the last bit, which can move a sample lying within
~1e-16 of a pixel edge.  The tests count such samples and require none at
these sizes."""
import numpy as np
import pytest

from conftest import bits_equal
from helpers import Case, oracle_map, map_from_oracle, stack_map

pytestmark = pytest.mark.gpu


def hp_case(orc, nside, nest, ncomp=3, tiled=False, nside_tile=None, active=None, **kw):
    return Case(orc, coord="CAR", ncomp=ncomp, tiled=tiled, hp=(nside, nest, nside_tile),
                active=active, **kw)


@pytest.mark.parametrize("nside,nest", [(64, False), (64, True), (1024, False), (1024, True)])
def test_pixels(orc, gpulib, nside, nest):
    c = hp_case(orc, nside, nest, n_det=8, n_time=6000)
    got = np.array(c.eng.pixels(c.bore, c.dets, None))
    want = orc.pixels(c.pz, c.bore, c.dets, 1)
    assert np.count_nonzero(got != want) == 0


@pytest.mark.parametrize("nside_tile", [4, 16])
def test_pixels_tiled(orc, gpulib, nside_tile):
    c = hp_case(orc, 256, True, tiled=True, nside_tile=nside_tile, n_det=6, n_time=4000)
    got = np.array(c.eng.pixels(c.bore, c.dets, None))
    want = orc.pixels(c.pz, c.bore, c.dets, 2)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("nest", [False, True])
@pytest.mark.parametrize("ncomp", [1, 2, 3])
def test_projection(orc, gpulib, nest, ncomp):
    c = hp_case(orc, 128, nest, ncomp=ncomp, n_det=6, n_time=4000)
    m = c.blank((ncomp,))
    flat, offs = oracle_map(m)
    orc.to_map(c.pz, c.bore, c.dets, c.resp, c.signal, None, flat, offs)
    got = c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, None, None)
    scale = np.abs(flat).max()
    assert np.abs(got.ravel() - flat).max() <= 1e-12 * scale
    w = c.blank((ncomp, ncomp))
    wf, wo = oracle_map(w)
    orc.to_weight_map(c.pz, c.bore, c.dets, c.resp, None, wf, wo)
    gw = c.eng.to_weight_map(None, c.bore, c.dets, c.resp, None, None)
    assert np.abs(gw.ravel() - wf).max() <= 1e-12 * np.abs(wf).max()
    src = c.random_map((ncomp,))
    sf, so = oracle_map(src)
    want = np.zeros((6, 4000), np.float32)
    orc.from_map(c.pz, c.bore, c.dets, c.resp, sf, want, so)
    got_sig = np.array(c.eng.from_map(src, c.bore, c.dets, c.resp, None))
    assert bits_equal(got_sig, want)


def test_tiled_is_nest_cut_into_tiles(orc, gpulib):
    nside, nt = 128, 8
    u = hp_case(orc, nside, True, n_det=6, n_time=4000)
    t = hp_case(orc, nside, True, tiled=True, nside_tile=nt, n_det=6, n_time=4000)
    hits = np.array(t.eng.tile_hits(t.bore, t.dets))
    active = list(np.nonzero(hits)[0])
    t = hp_case(orc, nside, True, tiled=True, nside_tile=nt, active=active, n_det=6,
                n_time=4000)
    mu = u.eng.to_map(None, u.bore, u.dets, u.resp, u.signal, None, None)
    mt = t.eng.to_map(None, t.bore, t.dets, t.resp, t.signal, None, None)
    nppt = 12 * nside ** 2 // (12 * nt ** 2)
    for i, tile in enumerate(mt):
        sl = mu[:, i * nppt:(i + 1) * nppt]
        if tile is None:
            assert np.all(sl == 0)
        else:
            np.testing.assert_allclose(tile, sl, rtol=1e-12, atol=1e-12)


def test_ring_tiled_rejected():
    import so3g_gb300
    with pytest.raises(ValueError, match="RING not supported"):
        so3g_gb300.ProjEng_HP_TQU_Tiled((64, 0, 4, None))
    with pytest.raises(ValueError, match="Invalid nside"):
        so3g_gb300.ProjEng_HP_TQU_NonTiled((100, 1, None, None))
