"""ProjEng_Precomp on the GPU: parity with the oracle, and with the
on-the-fly engine given the on-the-fly engine's own pointing_matrix (the
reference demo's "precomp == on-the-fly" invariant)."""
import numpy as np
import pytest

import so3g_gb300
from so3g_gb300 import _abi
from conftest import bits_equal
from helpers import Case, oracle_map, map_from_oracle, stack_map

pytestmark = pytest.mark.gpu


def interior(c, m):
    """Map without row and column 0 of the parent map (tiles reassembled)."""
    if not isinstance(m, list):
        return np.asarray(m)[..., 1:, 1:].ravel()
    e = c.eng
    ty, tx = e.tile_shape
    lead = next(t for t in m if t is not None).shape[:-2]
    full = np.zeros(lead + tuple(e.naxis))
    for i, t in enumerate(m):
        if t is not None:
            r, q = divmod(i, e.tile_grid[1])
            full[..., r * ty:r * ty + t.shape[-2], q * tx:q * tx + t.shape[-1]] = t
    return full[..., 1:, 1:].ravel()


@pytest.mark.parametrize("tiled", [False, True])
@pytest.mark.parametrize("ncomp", [1, 3])
def test_precomp_matches_on_the_fly(orc, gpulib, tiled, ncomp):
    """pointing_matrix uses GetPixel, which rejects x in (-1, 0); the Tiled
    on-the-fly projection uses GetPixels, which truncates it into column 0
    (src/Projection.cxx:1126-1129).  Row and column 0 of the parent map are
    therefore left out of the tiled comparison."""
    c = Case(orc, coord="CAR", ncomp=ncomp, tiled=tiled, n_det=5, n_time=4000)
    pix, proj = c.eng.pointing_matrix(c.bore, c.dets, c.resp, None, None)
    pix, proj = np.array(pix), np.array(proj)
    pe = (so3g_gb300.ProjEng_Precomp_Tiled if tiled else so3g_gb300.ProjEng_Precomp_NonTiled)()
    for accum in (_abi.ACCUM_ATOMIC, _abi.ACCUM_WARP_RUNS):
        m1 = pe.to_map(c.blank((ncomp,)), pix, proj, c.signal, None, None, accum=accum)
        m2 = c.eng.to_map(c.blank((ncomp,)), c.bore, c.dets, c.resp, c.signal, None, None)
        a, b = interior(c, m1), interior(c, m2)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
        w1 = pe.to_weight_map(c.blank((ncomp, ncomp)), pix, proj, None, None, accum=accum)
        w2 = c.eng.to_weight_map(c.blank((ncomp, ncomp)), c.bore, c.dets, c.resp, None, None)
        a, b = interior(c, w1), interior(c, w2)
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    src = c.random_map((ncomp,))
    s1 = np.array(pe.from_map(src, pix, proj, None))
    s2 = np.array(c.eng.from_map(src, c.bore, c.dets, c.resp, None))
    # Precomp sums the components in float32 before adding (:2073-2080),
    # on-the-fly adds each term to the float32 signal: equal to float32
    # rounding, on the samples pointing_matrix puts on the map.
    on = pix[..., 0] >= 0
    np.testing.assert_allclose(s1[on], s2[on], rtol=1e-5, atol=1e-5)
    assert np.all(s1[~on] == 0)


@pytest.mark.parametrize("tiled", [False, True])
def test_precomp_oracle(orc, gpulib, tiled):
    c = Case(orc, coord="ZEA", ncomp=3, tiled=tiled, n_det=4, n_time=3000)
    pix, proj = orc.pointing_matrix(c.pz, c.bore, c.dets, c.resp, c.eng.index_count)
    pe = (so3g_gb300.ProjEng_Precomp_Tiled if tiled else so3g_gb300.ProjEng_Precomp_NonTiled)()
    w = np.array([1., 0., 2., .5], np.float32)
    m = c.blank((3,))
    flat, offs = oracle_map(m)
    kw = {}
    if tiled:
        dims = np.array([t.shape[-2:] if t is not None else (0, 0) for t in m], np.int32)
        kw = dict(tile_offset=offs, tile_dims=dims)
    else:
        kw = dict(naxis=m.shape[-2:])
    orc.precomp_to_map(pix, proj, c.signal, w, flat, **kw)
    got = pe.to_map(m, pix, proj, c.signal, w, None)
    assert np.abs(stack_map(got) - flat).max() <= 1e-12 * np.abs(flat).max()
    src = c.random_map((3,))
    sf, so = oracle_map(src)
    want = np.zeros((4, 3000), np.float32)
    if tiled:
        orc.precomp_from_map(pix, proj, sf, want, tile_offset=so, tile_dims=kw["tile_dims"])
    else:
        orc.precomp_from_map(pix, proj, sf, want, naxis=src.shape[-2:])
    got_sig = np.array(pe.from_map(src, pix, proj, None))
    assert bits_equal(got_sig, want)


def test_precomp_pixel_out_of_range(orc, gpulib):
    pe = so3g_gb300.ProjEng_Precomp_NonTiled()
    pix = np.zeros((1, 10, 2), np.int32)
    pix[0, 3] = (2, 50)      # outside a (3, 4, 5) map
    proj = np.ones((1, 10, 3), np.float32)
    with pytest.raises(ValueError, match="out of range"):
        pe.to_map(np.zeros((3, 4, 5)), pix, proj, np.ones((1, 10), np.float32), None, None)


@pytest.mark.parametrize("n_time", [3000, 3004, 3001, 9000])
@pytest.mark.parametrize("ncomp", [1, 2, 3])
def test_precomp_vector_and_scalar_paths(orc, gpulib, n_time, ncomp):
    """n_time a multiple of 4 (16-byte aligned rows): the vectorised
    kernels, over one piece or several (9000 samples: pieces of 4096);
    otherwise the per-sample ones.  Both against the oracle: maps
    to float64 summation order, from_map into a non-zero signal bit for bit,
    with samples off the map (negative pixel) and detector weights."""
    import torch
    c = Case(orc, coord="CAR", ncomp=ncomp, tiled=False, n_det=6, n_time=n_time)
    pix, proj = orc.pointing_matrix(c.pz, c.bore, c.dets, c.resp, c.eng.index_count)
    pix[1, ::7, 0] = -1
    pe = so3g_gb300.ProjEng_Precomp_NonTiled()
    w = np.array([1., 0., 2., .5, 1.5, .25], np.float32)
    m = c.blank((ncomp,))
    naxis = m.shape[-2:]
    want = np.zeros_like(m)
    orc.precomp_to_map(pix, proj, c.signal, w, want, naxis=naxis)
    got = pe.to_map(m, pix, proj, c.signal, w, None)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    ww = np.zeros((ncomp,) + m.shape)
    orc.precomp_to_weight_map(pix, proj, w, ww, naxis=naxis)
    gw = pe.to_weight_map(np.zeros_like(ww), pix, proj, w, None)
    assert np.abs(gw - ww).max() <= 1e-12 * np.abs(ww).max()
    src = c.random_map((ncomp,))
    sig0 = np.random.default_rng(3).standard_normal((6, n_time)).astype(np.float32)
    want_s = sig0.copy()
    orc.precomp_from_map(pix, proj, src, want_s, naxis=naxis)
    got_s = np.array(pe.from_map(src, pix, proj, sig0.copy()))
    assert bits_equal(got_s, want_s)
    # Device tensors take the same kernels.
    dev = [torch.from_numpy(x).cuda() for x in (pix, proj, sig0.copy())]
    got_d = pe.from_map(torch.from_numpy(src).cuda(), *dev).cpu().numpy()
    assert bits_equal(got_d, want_s)


def test_precomp_pixel_out_of_range_vectorised(orc, gpulib):
    pe = so3g_gb300.ProjEng_Precomp_NonTiled()
    pix = np.zeros((2, 16, 2), np.int32)
    pix[1, 5] = (4, 0)      # row 4 of a (3, 4, 5) map
    proj = np.ones((2, 16, 3), np.float32)
    with pytest.raises(ValueError, match="out of range"):
        pe.to_map(np.zeros((3, 4, 5)), pix, proj, np.ones((2, 16), np.float32), None, None)
    with pytest.raises(ValueError, match="out of range"):
        pe.from_map(np.zeros((3, 4, 5)), pix, proj, None)
