"""Pointing parity on the GPU: coords, pixels and pointing_matrix of the
CUDA library against the CPU oracle, bit for bit."""
import numpy as np
import pytest

from conftest import bits_equal
from helpers import COORDS, Case

pytestmark = pytest.mark.gpu

# Coordinate systems whose coords() use only + - * / sqrt and the tables:
# bit-exact.  CEA calls the math-library atan2 (src/Projection.cxx:468),
# which CUDA and the host libm may round differently in the last bit.
EXACT = [c for c in COORDS if c != "CEA"]


@pytest.mark.parametrize("coord", COORDS)
def test_coords(orc, gpulib, coord):
    c = Case(orc, coord=coord, n_det=6, n_time=5000)
    got = np.array(c.eng.coords(c.bore, c.dets, None))
    want = orc.coords(c.pz, c.bore, c.dets)
    assert got.shape == want.shape
    if coord in EXACT:
        assert bits_equal(got, want)
    else:
        # CEA: the longitude is the math library's atan2 -- CUDA's and the
        # host's may round differently in the last bit.  Counted; every
        # other coordinate must be bit-identical.
        diff = got.view(np.int64) != want.view(np.int64)
        n_lon = int(np.count_nonzero(diff[..., 0]))
        print("CEA coords: %d of %d longitudes differ in the last bit" % (n_lon, diff[..., 0].size))
        assert not diff[..., 1:].any()
        np.testing.assert_allclose(got[..., 0], want[..., 0], rtol=4e-16, atol=1e-15)


@pytest.mark.parametrize("coord", COORDS)
@pytest.mark.parametrize("tiled", [False, True])
def test_pixels(orc, gpulib, coord, tiled):
    c = Case(orc, coord=coord, tiled=tiled, n_det=6, n_time=5000)
    got = np.array(c.eng.pixels(c.bore, c.dets, None))
    want = orc.pixels(c.pz, c.bore, c.dets, c.eng.index_count)
    assert got.shape == want.shape
    # Some samples are off the map, so the carried ("stale") slots are
    # exercised too.
    assert (want[..., 0] == -1).any() and (want[..., 0] >= 0).any()
    # CEA's last-bit atan2 differences move a pixel only for a sample within
    # ~1e-16 of a pixel edge: the count must be 0 here as for the others.
    n_bad = int(np.count_nonzero(np.any(got != want, axis=-1)))
    print("%s pixels: %d of %d samples differ" % (coord, n_bad, got.shape[0] * got.shape[1]))
    assert n_bad == 0


@pytest.mark.parametrize("coord", COORDS)
@pytest.mark.parametrize("ncomp", [1, 2, 3])
@pytest.mark.parametrize("tiled", [False, True])
def test_pointing_matrix(orc, gpulib, coord, ncomp, tiled):
    c = Case(orc, coord=coord, ncomp=ncomp, tiled=tiled, n_det=4, n_time=3000)
    pix, proj = c.eng.pointing_matrix(c.bore, c.dets, c.resp, None, None)
    wpix, wproj = orc.pointing_matrix(c.pz, c.bore, c.dets, c.resp, c.eng.index_count)
    assert np.array_equal(np.array(pix), wpix)
    assert bits_equal(np.array(proj), wproj)


def test_pixels_long_offmap_stretch(orc, gpulib):
    """Stale slots carried across many warp sub-ranges and blocks: a
    detector off the map for most of a long timeline."""
    c = Case(orc, coord="CAR", tiled=True, n_det=3, n_time=70000, seed=5)
    got = np.array(c.eng.pixels(c.bore, c.dets, None))
    want = orc.pixels(c.pz, c.bore, c.dets, c.eng.index_count)
    assert np.array_equal(got, want)


def test_outputs_into_given_buffers(orc, gpulib):
    c = Case(orc, coord="CAR", n_det=3, n_time=1000)
    out = np.full((3, 1000, 4), np.nan)
    ret = c.eng.coords(c.bore, c.dets, out)
    assert all(np.shares_memory(r, out) for r in ret)
    assert bits_equal(out, orc.coords(c.pz, c.bore, c.dets))
    rows = [np.zeros((1000, 2), np.int32) for _ in range(3)]
    ret = c.eng.pixels(c.bore, c.dets, rows)
    assert ret is rows
    assert np.array_equal(np.array(rows), orc.pixels(c.pz, c.bore, c.dets, 2))


def test_device_tensors(orc, gpulib):
    import torch
    c = Case(orc, coord="TAN", n_det=4, n_time=2000)
    b = torch.from_numpy(c.bore).cuda()
    d = torch.from_numpy(c.dets).cuda()
    out = c.eng.coords(b, d, None)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    assert bits_equal(out.cpu().numpy(), orc.coords(c.pz, c.bore, c.dets))
