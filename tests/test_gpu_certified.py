"""The certified double-float pointing (CAR, nearest-neighbour flat maps)
against the exact float64 pointing on the GPU, sample by sample.

from_map with maps built to read back one quantity per sample exposes
every pixel index and every float32 spin factor: a map holding each
pixel's own index in its T plane returns the pixel of every sample
(exactly representable in float32 here), and maps with Q = 1 or U = 1 return
the spin factors.  The certified path must reproduce the exact path's
values bit for bit, at scale and on inputs placed on pixel edges, at the
atan2 seam, near the native poles and at polarisation angles where a spin
factor vanishes."""
import numpy as np
import pytest

from so3g_gb300 import _abi, synth
from conftest import bits_equal

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60


def _engine(shape, res, tiled, ncomp=3):
    tile = (64, 96) if tiled else None
    p = synth.car_projectionist(shape, res, tile_shape=tile)
    return p, p.get_ProjEng({1: "T", 2: "QU", 3: "TQU"}[ncomp])


def _probe_maps(eng, tiled, ncomp):
    """Maps whose from_map returns (pixel index, pf[1], pf[2]) per sample."""
    import torch
    shape = eng._pix_shape() if not tiled else None

    def mk(fill):
        if not tiled:
            m = np.zeros((ncomp,) + shape)
            fill(m, 0, 0)
            return torch.from_numpy(m).cuda()
        out = []
        for i in range(eng._n_tile()):
            ty, tx = eng._tile_pix_shape(i)
            r, q = divmod(i, eng.tile_grid[1])
            m = np.zeros((ncomp, ty, tx))
            fill(m, r * eng.tile_shape[0], q * eng.tile_shape[1])
            out.append(torch.from_numpy(m).cuda())
        return out

    def pixel_index(m, y0, x0):
        iy, ix = np.meshgrid(np.arange(m.shape[1]) + y0, np.arange(m.shape[2]) + x0,
                             indexing="ij")
        m[0] = 1 + iy * 4096 + ix

    maps = [mk(pixel_index)]
    for k in range(1, ncomp):
        def one(m, y0, x0, k=k):
            m[k] = 1.0
        maps.append(mk(one))
    return maps


def _compare(eng, q, dets, resp, tiled, ncomp):
    import torch
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    maps = _probe_maps(eng, tiled, ncomp)
    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        res = []
        for m in maps:
            sig = eng.from_map(m, qd, dd, rd, None)
            res.append(sig.cpu().numpy())
        out[mode] = res
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
        assert bits_equal(a, b)
    return out[_abi.POINTING_EXACT]


@pytest.mark.parametrize("tiled", [False, True])
def test_certified_equals_exact_at_scale(tiled):
    Q, dets, resp, gamma, _ = synth.workload(200, 100_000, seed=11, radius_deg=1.5)
    p, eng = _engine((700, 900), ARCMIN, tiled)
    q = synth.native(p, Q)
    res = _compare(eng, q, dets, resp, tiled, 3)
    on = res[0] > 0
    assert 0.5 < on.mean() < 1.0        # on and off the map
    # The spin factors span [-1, 1].
    assert res[1][on].min() < -0.99 and res[1][on].max() > 0.99


def test_certified_from_map_accumulation_values():
    """from_map adds map*pf to the signal in float64 and rounds to float32
    after every term; the certified path reproduces that for signed zeros,
    tiny and huge map values and a non-zero starting signal."""
    import torch
    Q, dets, resp, gamma, _ = synth.workload(16, 50_000, seed=13, radius_deg=0.5)
    p, eng = _engine((300, 400), ARCMIN, False)
    q = synth.native(p, Q)
    rng = np.random.default_rng(3)
    m = rng.standard_normal((3, 300, 400))
    pick = rng.random(m.shape)
    m[pick < 0.05] = 0.0
    m[(pick >= 0.05) & (pick < 0.1)] = -0.0
    m[(pick >= 0.1) & (pick < 0.15)] *= 1e-30
    m[(pick >= 0.15) & (pick < 0.2)] *= 1e30
    m[(pick >= 0.2) & (pick < 0.25)] = np.round(m[(pick >= 0.2) & (pick < 0.25)] * 8) / 8
    sig0 = rng.standard_normal((16, 50_000)).astype(np.float32)
    sig0[:, ::7] = 0.0
    sig0[:, 1::7] = -0.0
    qd, dd, rd, md = (torch.from_numpy(x).cuda() for x in (q, dets, resp, m))
    out = []
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        s = torch.from_numpy(sig0.copy()).cuda()
        eng.from_map(md, qd, dd, rd, s)
        out.append(s.cpu().numpy())
    assert bits_equal(out[0], out[1])


def test_certified_to_map_matches_exact():
    import torch
    Q, dets, resp, gamma, sig = synth.workload(64, 100_000, seed=12, radius_deg=1.0)
    p, eng = _engine((600, 600), ARCMIN, False)
    q = synth.native(p, Q)
    qd, dd, rd, sd = (torch.from_numpy(x).cuda() for x in (q, dets, resp, sig))
    maps = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        m = eng.to_map(None, qd, dd, rd, sd, None, None)
        w = eng.to_weight_map(None, qd, dd, rd, None, None)
        maps[mode] = (m.cpu().numpy(), w.cpu().numpy())
    for a, b in zip(maps[_abi.POINTING_EXACT], maps[_abi.POINTING_CERTIFIED]):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def _quats_at(lon, lat, gamma):
    """Native-frame pointing quaternions at (lon, lat) with angle gamma."""
    from so3g_gb300.proj import quat
    return np.ascontiguousarray(np.asarray(quat.rotation_lonlat(lon, lat, gamma)))


@pytest.mark.parametrize("ncomp", [1, 2, 3])
def test_certified_edge_cases(ncomp):
    rng = np.random.default_rng(5)
    p, eng = _engine((300, 400), 0.5 * ARCMIN, False, ncomp=ncomp)
    ny, nx, dy, dx, cry, crx = eng.naxis + eng.cdelt + eng.crpix
    n = 40000
    # Pixel edges: x and y exactly on integer pixel coordinates (and 1e-13
    # either side), plus the map's outer edges.
    ix = rng.integers(-2, nx + 2, n).astype(float)
    iy = rng.integers(-2, ny + 2, n).astype(float)
    jit = rng.choice([0., 1e-13, -1e-13, 1e-9, 0.5], n)
    lon = (ix + jit - crx + 1 - 0.5) * dx
    lat = (iy + jit - cry + 1 - 0.5) * dy
    # Polarisation angles where pf1 or pf2 vanish, and random ones.
    gam = rng.choice([0., np.pi / 4, np.pi / 2, -np.pi / 4, np.pi / 8], n) + \
        rng.choice([0., 1e-9, rng.uniform(0, np.pi)], n)
    q = _quats_at(lon, lat, gam)
    # Detector at the boresight (identity offset).
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    _compare(eng, q, dets, resp, False, ncomp)


def test_certified_seam_and_poles():
    """Samples at the +-pi longitude seam and close to the native poles are
    recomputed exactly; results stay equal."""
    p, eng = _engine((200, 200), 60 * ARCMIN, False)
    n = 20000
    rng = np.random.default_rng(9)
    lon = np.concatenate([np.pi - rng.uniform(0, 1e-9, n // 4), -np.pi + rng.uniform(0, 1e-9, n // 4),
                          rng.uniform(-np.pi, np.pi, n // 2)])
    lat = np.concatenate([rng.uniform(-0.1, 0.1, n // 2),
                          rng.choice([1, -1], n // 2) * rng.uniform(1.5, np.pi / 2, n // 2)])
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.]])
    resp = np.ones((1, 2), np.float32)
    # A map spanning 200 deg so that the seam region is on the map.
    eng2 = type(eng)((200, 200, 1.8 * np.pi / 180, -1.8 * np.pi / 180, 100.5, 100.5))
    _compare(eng2, q, dets, resp, False, 3)
