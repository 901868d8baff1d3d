"""Seeded random sweep of the certified and mixed pointing against the
exact float64 path: random projections, resolutions, map sizes, tilings,
scan elevations and speeds, focal-plane radii and map centres offset from
the scan.  from_map of probe maps reads back every sample's pixel index
(T = 1 + index, exact in float32) and spin factors (Q = 1, U = 1): pixel
indices must be bit-identical in both modes, spin factors bit-identical in
the certified mode and within float32 evaluation error in the mixed
mode."""
import numpy as np
import pytest

from conftest import bits_equal
from so3g_gb300 import _abi, synth
from test_gpu_certified import _hp_engine, _hp_probe_maps, _probe_maps

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60
MODES = (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED, _abi.POINTING_MIXED)


def _case(seed, kinds=("CAR", "TAN", "ZEA", "SIN", "HP", "ARC")):
    rng = np.random.default_rng(1000 + seed)
    kind = kinds[seed % len(kinds)]
    el = float(rng.uniform(20., 75.))
    az0 = float(rng.uniform(0., 360.))
    n_det = 8
    n_time = 20000
    Q, dets, resp, gamma, _ = synth.workload(
        n_det, n_time, seed=seed, radius_deg=float(rng.uniform(0.2, 4.)),
        rate=float(rng.choice([50., 200.])), el=el, az0=az0,
        throw=float(rng.uniform(1., 30.)), v_az=float(rng.uniform(0.3, 3.)), signal=False)
    resp = resp.copy()
    resp[:, 1] = rng.uniform(0.3, 1.0, n_det).astype(np.float32)
    if kind == "HP":
        nside = int(rng.choice([64, 256, 1024]))
        nest = bool(rng.integers(0, 2))
        tiled = nest and bool(rng.integers(0, 2))
        if len(kinds) == 2 and nest:   # the chunked sweep tiles every NEST map
            tiled = True
        p, eng = _hp_engine(nside, nest, tiled)
        maps = _hp_probe_maps(eng, tiled, 3)
    else:
        res = float(rng.choice([0.25, 0.5, 1., 3.])) * ARCMIN
        ny, nx = (int(rng.integers(200, 1500)), int(rng.integers(200, 1500)))
        tiled = bool(rng.integers(0, 2))
        tile = (int(rng.integers(16, 200)), int(rng.integers(16, 200))) if tiled else None
        # Map centre near, not on, the scan centre.
        p = synth.car_projectionist((ny, nx), res, el=el + float(rng.uniform(-1, 1)),
                                    az0=az0 + float(rng.uniform(-1, 1)), proj=kind,
                                    tile_shape=tile)
        eng = p.get_ProjEng("TQU")
        maps = _probe_maps(eng, tiled, 3)
    q = synth.native(p, Q)
    return kind, eng, maps, q, dets, resp


@pytest.mark.parametrize("seed", range(36))
def test_random_geometry(gpulib, seed):
    _check_geometry(_case(seed))


@pytest.mark.parametrize("seed", range(100, 124))
def test_random_geometry_chunked(gpulib, seed):
    """The same sweep over the geometries the chunked mixed kernels take
    (CAR and HEALPix, untiled and tiled, ragged edge tiles)."""
    _check_geometry(_case(seed, kinds=("CAR", "HP")))


def _check_geometry(case):
    import torch
    kind, eng, maps, q, dets, resp = case
    qd, dd, rd = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (q, dets, resp))
    out = {}
    for mode in MODES:
        eng.pointing = mode
        out[mode] = [eng.from_map(m, qd, dd, rd, None).cpu().numpy() for m in maps]
    ex = out[_abi.POINTING_EXACT]
    assert (ex[0] > 0).any(), "no sample on the map"
    for a, b in zip(ex, out[_abi.POINTING_CERTIFIED]):
        assert bits_equal(a, b)
    mx = out[_abi.POINTING_MIXED]
    assert bits_equal(ex[0], mx[0])
    for a, b in zip(ex[1:], mx[1:]):
        assert np.abs(a - b).max() <= 2e-5


@pytest.mark.parametrize("seed", range(0, 36, 3))
def test_random_geometry_to_map(gpulib, seed):
    """to_map over the same random geometries: certified maps equal the
    float64 path's up to float64 summation order, mixed ones within 1e-6
    of the scale."""
    import torch
    kind, eng, maps, q, dets, resp = _case(seed)
    rng = np.random.default_rng(seed)
    sig = torch.from_numpy(rng.standard_normal((len(dets), len(q)), dtype=np.float32)).cuda()
    qd, dd, rd = (torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (q, dets, resp))

    def flat(m):
        if isinstance(m, list):
            return np.concatenate([t.cpu().numpy().ravel() for t in m if t is not None])
        return m.cpu().numpy().ravel()
    out = {}
    for mode in MODES:
        eng.pointing = mode
        out[mode] = flat(eng.to_map(None, qd, dd, rd, sig, None, None))
    ex = out[_abi.POINTING_EXACT]
    scale = np.abs(ex).max()
    assert scale > 0
    assert np.abs(out[_abi.POINTING_CERTIFIED] - ex).max() <= 1e-12 * scale
    assert np.abs(out[_abi.POINTING_MIXED] - ex).max() <= 1e-6 * scale
