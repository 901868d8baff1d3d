"""The certified double-float pointing (CAR, TAN, ZEA and SIN with flat
pixelizors) against the exact float64 pointing on the GPU, sample by
sample.

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


def _engine(shape, res, tiled, ncomp=3, proj="CAR", interpol=None):
    tile = (64, 96) if tiled else None
    p = synth.car_projectionist(shape, res, tile_shape=tile, proj=proj, interpol=interpol)
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


@pytest.mark.parametrize("proj", ["TAN", "ZEA", "SIN", "ARC"])
@pytest.mark.parametrize("tiled", [False, True])
def test_certified_zenithal_at_scale(proj, tiled):
    """Nearest-neighbour zenithal maps: every pixel index and spin factor
    equal, on fine pixels (0.25 arcmin) so that many samples fall close to
    pixel edges."""
    Q, dets, resp, gamma, _ = synth.workload(100, 100_000, seed=21, radius_deg=1.0)
    p, eng = _engine((900, 1100), 0.25 * ARCMIN, tiled, proj=proj)
    q = synth.native(p, Q)
    res = _compare(eng, q, dets, resp, tiled, 3)
    on = res[0] > 0
    assert 0.2 < on.mean() < 1.0
    assert res[1][on].min() < -0.99 and res[1][on].max() > 0.99


def _solve_lonlat(orc, eng, x_t, y_t, lon0, lat0, gam):
    """(lon, lat) whose exact pixel coordinates are (x_t, y_t): Newton's
    method on the oracle's float64 coordinates."""
    pz = eng._pz()
    pz.pointing = _abi.POINTING_EXACT
    (ny, nx), (dy, dx), (cry, crx) = eng.naxis, eng.cdelt, eng.crpix
    lon, lat = lon0.copy(), lat0.copy()
    one = np.array([[1., 0., 0., 0.]])
    h = 1e-7

    def pixel_xy(lo, la):
        c = orc.coords(pz, _quats_at(lo, la, gam), one)[0]
        return c[:, 0] / dx + crx - 1 + 0.5, c[:, 1] / dy + cry - 1 + 0.5

    for _ in range(6):
        # Points at the projection's pole have a singular Jacobian: their
        # NaN coordinates make samples that fall off the map.
        with np.errstate(invalid="ignore", divide="ignore"):
            lon, lat = _newton_step(pixel_xy, lon, lat, x_t, y_t, h)
    return lon, lat


def _newton_step(pixel_xy, lon, lat, x_t, y_t, h):
    """One Newton step towards pixel coordinates (x_t, y_t)."""
    x, y = pixel_xy(lon, lat)
    xa, ya = pixel_xy(lon + h, lat)
    xb, yb = pixel_xy(lon, lat + h)
    j11, j21 = (xa - x) / h, (ya - y) / h
    j12, j22 = (xb - x) / h, (yb - y) / h
    det = j11 * j22 - j12 * j21
    ex, ey = x_t - x, y_t - y
    return lon + (j22 * ex - j12 * ey) / det, lat + (-j21 * ex + j11 * ey) / det


@pytest.mark.parametrize("proj", ["TAN", "ZEA", "SIN", "ARC"])
def test_certified_zenithal_edges(orc, proj):
    """Zenithal samples placed on pixel edges (and 1e-13 either side): the
    uncertain ones go to the exact path and all results stay equal."""
    rng = np.random.default_rng(17)
    p, eng = _engine((300, 400), 0.5 * ARCMIN, False, proj=proj)
    (ny, nx) = eng.naxis
    n = 20000
    ix = rng.integers(-2, nx + 2, n).astype(float)
    iy = rng.integers(-2, ny + 2, n).astype(float)
    jit = rng.choice([0., 1e-13, -1e-13, 1e-9, 0.5], n)
    gam = rng.choice([0., np.pi / 4, np.pi / 8], n) + rng.choice([0., 1e-9, 0.3], n)
    # Start from the small-angle inverse of the projection about the
    # native pole (the map centre).
    (dy, dx), (cry, crx) = eng.cdelt, eng.crpix
    u = (ix + jit - (crx - 0.5)) * abs(dx)
    v = (iy + jit - (cry - 0.5)) * dy
    lon0 = np.arctan2(u, v)
    lat0 = np.pi / 2 - np.hypot(u, v)
    lon, lat = _solve_lonlat(orc, eng, ix + jit, iy + jit, lon0, lat0, gam)
    q = _quats_at(lon, lat, gam)
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    res = _compare(eng, q, dets, resp, False, 3)
    assert (res[0][0] > 0).mean() > 0.5


@pytest.mark.parametrize("proj", ["CAR", "TAN", "ZEA"])
@pytest.mark.parametrize("tiled", [False, True])
def test_certified_bilinear(proj, tiled):
    """Bilinear maps: the certified path takes the same taps and the same
    spin factors; its interpolation weights are within one float32 ulp of
    the exact path's.  Maps and signals agree to 1e-6 of their largest
    value."""
    import torch
    Q, dets, resp, gamma, sig = synth.workload(64, 100_000, seed=23, radius_deg=1.0)
    p, eng = _engine((500, 600), ARCMIN, tiled, proj=proj, interpol="bilinear")
    q = synth.native(p, Q)
    qd, dd, rd, sd = (torch.from_numpy(x).cuda() for x in (q, dets, resp, sig))
    def zeros(lead):
        if not tiled:
            return torch.zeros(lead + eng._pix_shape(), dtype=torch.float64, device="cuda")
        return [torch.zeros(lead + eng._tile_pix_shape(i), dtype=torch.float64, device="cuda")
                for i in range(eng._n_tile())]

    def flat(x):
        if isinstance(x, list):
            x = torch.cat([t.reshape(-1) for t in x])
        return x.reshape(-1).double().cpu().numpy()

    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        m = eng.to_map(zeros((3,)), qd, dd, rd, sd, None, None)
        w = eng.to_weight_map(zeros((3, 3)), qd, dd, rd, None, None)
        back = eng.from_map(m, qd, dd, rd, None)
        out[mode] = [flat(x) for x in (m, w, back)]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()


def _hp_engine(nside, nest, tiled, ncomp=3):
    from so3g_gb300.proj.wcs import ProjectionistHealpix
    if tiled:
        nt = 12 * 4 ** 2
        p = ProjectionistHealpix.for_healpix(nside, nside_tile=4, active_tiles=list(range(nt)),
                                             ordering="NEST")
    else:
        p = ProjectionistHealpix.for_healpix(nside, ordering="NEST" if nest else "RING")
    return p, p.get_ProjEng({1: "T", 2: "QU", 3: "TQU"}[ncomp])


def _hp_probe_maps(eng, tiled, ncomp):
    import torch
    if not tiled:
        npix = eng._pix_shape()[0]
        m = np.zeros((ncomp, npix))
        m[0] = 1 + np.arange(npix)
        maps = [torch.from_numpy(m).cuda()]
        for k in range(1, ncomp):
            mk = np.zeros((ncomp, npix))
            mk[k] = 1.0
            maps.append(torch.from_numpy(mk).cuda())
        return maps
    nppt = eng._tile_pix_shape(0)[0]
    out = []
    for k in range(ncomp):
        tiles = []
        for i in range(eng._n_tile()):
            t = np.zeros((ncomp, nppt))
            t[k] = (1 + i * nppt + np.arange(nppt)) if k == 0 else 1.0
            tiles.append(torch.from_numpy(t).cuda())
        out.append(tiles)
    return out


@pytest.mark.parametrize("nside,nest,tiled", [(64, False, False), (1024, False, False),
                                              (1024, True, False), (512, True, True),
                                              (4096, False, False)])
def test_certified_healpix_at_scale(nside, nest, tiled):
    """HEALPix: pixel indices and spin factors of the certified path equal
    the exact path's, over a scan that crosses the polar caps, the
    equatorial belt and phi = 0 (pixel values up to 2^24 are exact in
    float32, so larger maps are probed through index mod 2^22)."""
    import torch
    # Two scans: one across the belt/cap boundary (el ~ 41.8 deg) and the
    # +-pi seam of phi, one in the northern cap across phi = 0.
    Q1, dets, resp, gamma, _ = synth.workload(100, 30_000, seed=41, radius_deg=2.0, el=40.,
                                              throw=60., v_az=3.)
    Q2, _, _, _, _ = synth.workload(100, 30_000, seed=41, radius_deg=2.0, el=65., az0=0.,
                                    throw=60., v_az=3.)
    Q = np.concatenate([Q1, Q2])
    p, eng = _hp_engine(nside, nest, tiled)
    q = synth.native(p, Q)
    maps = _hp_probe_maps(eng, tiled, 3)
    if not tiled and 12 * nside * nside >= 1 << 24:
        m0 = maps[0].cpu().numpy()
        m0[0] = 1 + np.arange(m0.shape[1]) % (1 << 22)
        maps[0] = torch.from_numpy(m0).cuda()
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        out[mode] = [eng.from_map(m, qd, dd, rd, None).cpu().numpy() for m in maps]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
        assert bits_equal(a, b)


def test_certified_healpix_edges(orc):
    """HEALPix samples on the equatorial/polar boundary (|z| = 2/3), at
    phi = 0 and +-pi, and on in-face pixel edges of the equatorial belt."""
    import torch
    rng = np.random.default_rng(43)
    nside = 256
    n = 30000
    z_edge = rng.choice([2 / 3, -2 / 3], n // 3) + rng.choice([0., 1e-15, -1e-15, 1e-12], n // 3)
    lat_a = np.arcsin(z_edge)
    lon_a = rng.uniform(-np.pi, np.pi, n // 3)
    lat_b = rng.uniform(-1.2, 1.2, n // 3)
    lon_b = rng.choice([0., np.pi, -np.pi], n // 3) + rng.choice([0., 1e-15, -1e-15, 1e-9],
                                                                    n // 3)
    # Equatorial in-face edges: jp = 0.5 + tt - 0.75 z and jm = 0.5 + tt + 0.75 z
    # at multiples of 1/nside.
    k = n - 2 * (n // 3)
    jp = rng.integers(1, 4 * nside, k) / nside
    jm = jp + rng.integers(-nside // 2, nside // 2, k) / nside
    z = (jm - jp) / 1.5
    tt = (jp + jm) / 2 - 0.5
    ok = np.abs(z) < 0.66
    lat_c = np.arcsin(z[ok])
    lon_c = tt[ok] / 4 * 2 * np.pi
    lon_c = np.where(lon_c > np.pi, lon_c - 2 * np.pi, lon_c)
    lat = np.concatenate([lat_a, lat_b, lat_c])
    lon = np.concatenate([lon_a, lon_b, lon_c])
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, len(lat)))
    dets = np.array([[1., 0., 0., 0.]])
    resp = np.ones((1, 2), np.float32)
    for nest in (False, True):
        p, eng = _hp_engine(nside, nest, False)
        maps = _hp_probe_maps(eng, False, 3)
        qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
        out = {}
        for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
            eng.pointing = mode
            out[mode] = [eng.from_map(m, qd, dd, rd, None).cpu().numpy() for m in maps]
        for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
            assert bits_equal(a, b)


def test_certified_octant_boundaries():
    """CAR samples with |Y| = |X| in the atan2 of the longitude (lon =
    +-pi/4, +-3pi/4), where the table is read at its last knot."""
    n = 20000
    rng = np.random.default_rng(47)
    lon = rng.choice([np.pi / 4, -np.pi / 4, 3 * np.pi / 4, -3 * np.pi / 4], n) + \
        rng.choice([0., 1e-15, -1e-15, 1e-12], n)
    lat = rng.uniform(-1.3, 1.3, n)
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.]])
    resp = np.ones((1, 2), np.float32)
    p, eng = _engine((200, 200), 60 * ARCMIN, False)
    # 0.9 deg pixels over 360 deg x 180 deg, so that all four lons are on the map.
    eng2 = type(eng)((200, 400, 0.9 * np.pi / 180, -0.9 * np.pi / 180, 100.5, 200.5))
    res = _compare(eng2, q, dets, resp, False, 3)
    assert (res[0] > 0).mean() > 0.9


def _np(x):
    """A result (tensor, array or list of per-detector rows) as one array."""
    if isinstance(x, (list, tuple)):
        return np.stack([_np(e) for e in x])
    if hasattr(x, "cpu"):
        return x.cpu().numpy()
    return np.asarray(x)


def _edge_quats(orc, eng, proj, n, seed):
    """Native pointings on pixel edges (0, +-1e-13, 1e-9 and mid-pixel),
    the map's outer edges and the x in (-1, 0) strip, with polarisation
    angles where a spin factor vanishes (zenithal projections: solved for
    those pixel coordinates by Newton's method)."""
    rng = np.random.default_rng(seed)
    ny, nx, dy, dx, cry, crx = eng.naxis + eng.cdelt + eng.crpix
    ix = rng.integers(-2, nx + 2, n).astype(float)
    iy = rng.integers(-2, ny + 2, n).astype(float)
    jit = rng.choice([0., 1e-13, -1e-13, 1e-9, 0.5, -0.5], n)
    gam = rng.choice([0., np.pi / 4, np.pi / 2, -np.pi / 4], n) + \
        rng.choice([0., 1e-9, rng.uniform(0, np.pi)], n)
    if proj == "CAR":
        lon = (ix + jit - crx + 1 - 0.5) * dx
        lat = (iy + jit - cry + 1 - 0.5) * dy
    else:
        u = (ix + jit - (crx - 0.5)) * abs(dx)
        v = (iy + jit - (cry - 0.5)) * dy
        lon, lat = _solve_lonlat(orc, eng, ix + jit, iy + jit, np.arctan2(u, v),
                                 np.pi / 2 - np.hypot(u, v), gam)
    return _quats_at(lon, lat, gam)


@pytest.mark.parametrize("proj", ["CAR", "TAN", "ZEA", "SIN"])
@pytest.mark.parametrize("tiled,interpol", [(False, None), (True, None), (False, "bilinear"),
                                            (True, "bilinear")])
def test_certified_pixels_and_pointing_matrix(orc, proj, tiled, interpol):
    """pixels() and pointing_matrix() take the certified pointing (GetPixel
    of every flat pixelizor is the [0, n)-bounded nearest pixel, spin
    factors certified): bit-identical to the exact path on edge inputs,
    including the stale slots of off-map samples."""
    import torch
    p, eng = _engine((300, 400), 0.5 * ARCMIN, tiled, proj=proj, interpol=interpol)
    q = _edge_quats(orc, eng, proj, 30000, 21)
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        pix = eng.pixels(qd, dd, None)
        pm_pix, pm_proj = eng.pointing_matrix(qd, dd, rd, None, None)
        out[mode] = [_np(x) for x in (pix, pm_pix, pm_proj)]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
        assert bits_equal(a, b)
    # The inputs do land off the map and on it.
    assert (out[_abi.POINTING_EXACT][0][..., 0] == -1).any()
    assert (out[_abi.POINTING_EXACT][0][..., 0] >= 0).any()


@pytest.mark.parametrize("nest,tiled", [(False, False), (True, False), (True, True)])
def test_certified_healpix_pointing_matrix(nest, tiled):
    import torch
    rng = np.random.default_rng(44)
    n = 30000
    z = rng.choice([2 / 3, -2 / 3], n) + rng.choice([0., 1e-15, -1e-15, 1e-12, 0.3], n)
    lat = np.arcsin(np.clip(z, -1, 1))
    lon = rng.uniform(-np.pi, np.pi, n)
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.]])
    resp = np.ones((1, 2), np.float32)
    p, eng = _hp_engine(256, nest, tiled)
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        pm_pix, pm_proj = eng.pointing_matrix(qd, dd, rd, None, None)
        out[mode] = [_np(x) for x in (pm_pix, pm_proj)]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]):
        assert bits_equal(a, b)


def _ranges_lists(R):
    """pixel_ranges / tile_ranges output as nested lists of interval arrays."""
    if hasattr(R, "ranges") and callable(getattr(R, "ranges")):
        return np.asarray(R.ranges()).tolist()
    if isinstance(R, (list, tuple)) or hasattr(R, "__iter__"):
        return [_ranges_lists(x) for x in R]
    return R


@pytest.mark.parametrize("proj", ["CAR", "TAN"])
@pytest.mark.parametrize("interpol", [None, "bilinear"])
def test_certified_tile_hits_and_ranges(orc, proj, interpol):
    """tile_hits, pixel_ranges and tile_ranges take the certified taps:
    identical to the exact path on pixel-edge inputs."""
    import torch
    p, eng = _engine((300, 400), 0.5 * ARCMIN, True, proj=proj, interpol=interpol)
    q = _edge_quats(orc, eng, proj, 30000, 23)
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    qd, dd = (torch.from_numpy(x).cuda() for x in (q, dets))
    out = {}
    for mode in (_abi.POINTING_EXACT, _abi.POINTING_CERTIFIED):
        eng.pointing = mode
        hits = np.asarray(eng.tile_hits(qd, dd))
        pr = _ranges_lists(eng.pixel_ranges(qd, dd, None, 4))
        groups = [[i for i in range(len(hits)) if hits[i] and i % 3 == g] for g in range(3)]
        tr = _ranges_lists(eng.tile_ranges(qd, dd, groups))
        out[mode] = (hits, pr, tr)
    ex, ce = out[_abi.POINTING_EXACT], out[_abi.POINTING_CERTIFIED]
    assert np.array_equal(ex[0], ce[0]) and ex[0].sum() > 0
    assert ex[1] == ce[1]
    assert ex[2] == ce[2]
