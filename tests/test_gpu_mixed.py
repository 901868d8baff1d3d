"""Mixed-precision pointing (POINTING_MIXED: CAR, TAN, ZEA and SIN nearest
neighbour, and HEALPix): pixel indices bit-identical to the exact float64 path, sample by sample and on
pixel edges; spin factors, maps and signals within the mixed-precision
tolerance (1e-6 of their scale) of the exact path."""
import numpy as np
import pytest

from so3g_gb300 import _abi, synth
from conftest import bits_equal
from test_gpu_certified import _engine, _probe_maps, _quats_at

pytestmark = pytest.mark.gpu
ARCMIN = np.pi / 180 / 60
MODES = (_abi.POINTING_EXACT, _abi.POINTING_MIXED)


# Spin-factor error bounds of the float32 tier, relative to P.  Anywhere
# the tier runs (|sin lat| < 0.9): PF_BOUND_GUARD, reached only near that
# guard; on scans near the native equator (the benchmark geometry): 1e-6.
PF_BOUND_GUARD = 2e-5
PF_BOUND_SCAN = 1e-6


def _probe(eng, q, dets, resp, tiled, ncomp=3, pf_bound=PF_BOUND_SCAN):
    import torch
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    maps = _probe_maps(eng, tiled, ncomp)
    out = {}
    for mode in MODES:
        eng.pointing = mode
        out[mode] = [eng.from_map(m, qd, dd, rd, None).cpu().numpy() for m in maps]
    ex, mx = out[_abi.POINTING_EXACT], out[_abi.POINTING_MIXED]
    # Pixel index (T probe: 1 + index, exact in float32): bit for bit.
    assert bits_equal(ex[0], mx[0])
    # Spin factors: float32 evaluations.
    for a, b in zip(ex[1:], mx[1:]):
        assert np.abs(a - b).max() <= pf_bound
        assert np.abs(a - b).mean() <= 2e-7
    return ex


@pytest.mark.parametrize("tiled", [False, True])
def test_mixed_pixels_at_scale(tiled):
    Q, dets, resp, gamma, _ = synth.workload(200, 100_000, seed=51, radius_deg=1.5)
    p, eng = _engine((700, 900), ARCMIN, tiled)
    q = synth.native(p, Q)
    res = _probe(eng, q, dets, resp, tiled)
    on = res[0] > 0
    assert 0.5 < on.mean() < 1.0


def test_mixed_pixel_edges():
    rng = np.random.default_rng(53)
    p, eng = _engine((300, 400), 0.5 * ARCMIN, False)
    ny, nx, dy, dx, cry, crx = eng.naxis + eng.cdelt + eng.crpix
    n = 40000
    ix = rng.integers(-2, nx + 2, n).astype(float)
    iy = rng.integers(-2, ny + 2, n).astype(float)
    jit = rng.choice([0., 1e-13, -1e-13, 1e-9, 1e-6, -1e-5, 0.5], n)
    lon = (ix + jit - crx + 1 - 0.5) * dx
    lat = (iy + jit - cry + 1 - 0.5) * dy
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    _probe(eng, q, dets, resp, False)


def test_mixed_wide_map_seam_and_caps():
    """A map spanning 360 x 180 degrees: the atan2 seam, the octants and
    the regions beyond the float32 tier's |sin lat| < 0.9 guard."""
    n = 40000
    rng = np.random.default_rng(55)
    lon = np.concatenate([rng.choice([np.pi, -np.pi, np.pi / 4, -3 * np.pi / 4], n // 2) +
                          rng.choice([0., 1e-12, -1e-12, 1e-7], n // 2),
                          rng.uniform(-np.pi, np.pi, n // 2)])
    lat = rng.uniform(-1.5, 1.5, n)
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.]])
    resp = np.ones((1, 2), np.float32)
    p, eng = _engine((200, 200), 60 * ARCMIN, False)
    eng2 = type(eng)((200, 400, 0.9 * np.pi / 180, -0.9 * np.pi / 180, 100.5, 200.5))
    _probe(eng2, q, dets, resp, False, pf_bound=PF_BOUND_GUARD)


@pytest.mark.parametrize("tiled", [False, True])
def test_mixed_maps_within_tolerance(tiled):
    import torch
    Q, dets, resp, gamma, sig = synth.workload(64, 100_000, seed=57, radius_deg=1.0)
    p, eng = _engine((600, 600), ARCMIN, tiled)
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
    m_exact = None
    for mode in MODES:
        eng.pointing = mode
        m = eng.to_map(zeros((3,)), qd, dd, rd, sd, None, None)
        w = eng.to_weight_map(zeros((3, 3)), qd, dd, rd, None, None)
        if m_exact is None:
            m_exact = m
        # from_map of the same (exact) map in both modes.
        s0 = torch.from_numpy(np.full(sig.shape, 0.25, np.float32)).cuda()
        back = eng.from_map(m_exact, qd, dd, rd, s0)
        out[mode] = [flat(x) for x in (m, w, back)]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_MIXED]):
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()


@pytest.mark.parametrize("pixelization", ["car", "hp_ring", "hp_nest"])
@pytest.mark.parametrize("ncomp", [1, 2, 3])
@pytest.mark.parametrize("accum", [_abi.ACCUM_WARP_RUNS, _abi.ACCUM_ATOMIC])
@pytest.mark.parametrize("path", ["chunked", "per_sample"])
def test_mixed_to_map_layouts(pixelization, ncomp, accum, path):
    """The mixed to_map / to_weight_map / from_map (CAR untiled nearest,
    HEALPix untiled), through the chunked kernels and through the
    per-sample tier that calls below the chunked threshold take, with
    signal rows that are not 16-byte aligned (a column slice of a wider
    array), an odd sample count (a partial last chunk and an odd chunk
    count per piece), detector weights with zeros, every component count
    and both accumulation modes, against the exact path.  The HEALPix scan
    crosses the belt / cap boundary (|z| = 2/3)."""
    import torch
    import so3g_gb300
    from test_gpu_certified import _hp_engine
    so3g_gb300.set_chunked_min_samples(0 if path == "chunked" else 1 << 62)
    n_det, n_time = 24, 30_001
    if pixelization == "car":
        Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=59, radius_deg=1.0)
        p, eng = _engine((600, 600), ARCMIN, False, ncomp=ncomp)
    else:
        Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=59, radius_deg=3.0,
                                                   el=41.5, throw=40., v_az=2.)
        p, eng = _hp_engine(512, pixelization == "hp_nest", False, ncomp=ncomp)
    q = synth.native(p, Q)
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    wide = torch.zeros((n_det, n_time + 1), dtype=torch.float32, device="cuda")
    wide[:, 1:] = torch.from_numpy(sig).cuda()
    sv = wide[:, 1:]
    assert sv.data_ptr() % 16 != 0 and sv.stride(0) == n_time + 1
    w = np.linspace(0., 2., n_det).astype(np.float32)
    w[7] = 0.
    wd = torch.from_numpy(w).cuda()
    shape = eng._pix_shape()
    out = {}
    for mode in MODES:
        eng.pointing = mode
        m = eng.to_map(torch.zeros((ncomp,) + shape, dtype=torch.float64, device="cuda"), qd, dd,
                       rd, sv, wd, None, accum=accum)
        ww = eng.to_weight_map(torch.zeros((ncomp, ncomp) + shape, dtype=torch.float64,
                                           device="cuda"), qd, dd, rd, wd, None, accum=accum)
        base = torch.full((n_det, n_time + 1), 0.5, dtype=torch.float32, device="cuda")
        back = eng.from_map(out[_abi.POINTING_EXACT][0] if out else m, qd, dd, rd, base[:, 1:])
        out[mode] = [m, ww, back]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_MIXED]):
        a, b = a.double().cpu().numpy(), b.double().cpu().numpy()
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()
    # The strided signal was read, not copied: the zero-weight detector adds
    # nothing, the others something.
    m = out[_abi.POINTING_MIXED][0]
    assert float(m.abs().sum()) > 0


@pytest.mark.parametrize("pixelization", ["hp", "car"])
@pytest.mark.parametrize("accum", [_abi.ACCUM_WARP_RUNS, _abi.ACCUM_ATOMIC])
def test_mixed_tiled_maps(pixelization, accum):
    """The chunked to_map / to_weight_map / from_map on tiled maps -- NEST
    (nside 512, nside_tile 4) and CAR (80 x 400 in 64 x 96 tiles, edge
    tiles smaller, the scan crossing the map's edges, where the tiled
    pixelizor's truncation keeps (-1, 0) in row / column 0): the run keys
    are parent-map pixels, each run's tile looked up when it is flushed.
    Unaligned signal rows, an odd sample count, against the exact path; a
    sample on an absent tile raises the tiling error in both directions."""
    import torch
    from test_gpu_certified import _hp_engine
    n_det, n_time = 24, 30_001
    if pixelization == "hp":
        Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=63, radius_deg=3.0,
                                                   el=41.5, throw=40., v_az=2.)
        p, eng = _hp_engine(512, True, True)
    else:
        Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=63, radius_deg=1.0)
        p, eng = _engine((80, 400), 1.6 * ARCMIN, True)
    q = synth.native(p, Q)
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    wide = torch.zeros((n_det, n_time + 1), dtype=torch.float32, device="cuda")
    wide[:, 1:] = torch.from_numpy(sig).cuda()
    sv = wide[:, 1:]
    n_tile = eng._n_tile()

    def tiles(lead, skip=()):
        return [None if i in skip else
                torch.zeros(lead + tuple(eng._tile_pix_shape(i)), dtype=torch.float64,
                            device="cuda")
                for i in range(n_tile)]

    def flat(x):
        return torch.cat([t.reshape(-1) for t in x]).double().cpu().numpy()

    out = {}
    for mode in MODES:
        eng.pointing = mode
        m = eng.to_map(tiles((3,)), qd, dd, rd, sv, None, None, accum=accum)
        ww = eng.to_weight_map(tiles((3, 3)), qd, dd, rd, None, None, accum=accum)
        base = torch.full((n_det, n_time + 1), 0.5, dtype=torch.float32, device="cuda")
        src = out[_abi.POINTING_EXACT][0] if out else m
        back = eng.from_map(src, qd, dd, rd, base[:, 1:])
        out[mode] = [m, ww, back]
    for a, b in zip(out[_abi.POINTING_EXACT], out[_abi.POINTING_MIXED]):
        a = flat(a) if isinstance(a, list) else a.double().cpu().numpy()
        b = flat(b) if isinstance(b, list) else b.double().cpu().numpy()
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()
    m_ex = out[_abi.POINTING_EXACT][0]
    hit = [i for i, t in enumerate(m_ex) if float(t.abs().sum()) > 0]
    assert len(hit) > 1
    eng.pointing = _abi.POINTING_MIXED
    gone = hit[len(hit) // 2]
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index %d\)" % gone):
        eng.to_map(tiles((3,), skip=(gone,)), qd, dd, rd, sv, None, None, accum=accum)
    src = [None if i == gone else t for i, t in enumerate(m_ex)]
    with pytest.raises(RuntimeError, match=r"Tiling problem \(index %d\)" % gone):
        eng.from_map(src, qd, dd, rd, None)


def _probe_hp(eng, q, dets, resp, tiled, pf_bound=PF_BOUND_GUARD):
    import torch
    from test_gpu_certified import _hp_probe_maps
    qd, dd, rd = (torch.from_numpy(x).cuda() for x in (q, dets, resp))
    maps = _hp_probe_maps(eng, tiled, 3)
    out = {}
    for mode in MODES:
        eng.pointing = mode
        out[mode] = [eng.from_map(m, qd, dd, rd, None).cpu().numpy() for m in maps]
    ex, mx = out[_abi.POINTING_EXACT], out[_abi.POINTING_MIXED]
    assert bits_equal(ex[0], mx[0])
    for a, b in zip(ex[1:], mx[1:]):
        assert np.abs(a - b).max() <= pf_bound
        assert np.abs(a - b).mean() <= 2e-7


@pytest.mark.parametrize("nside,nest,tiled", [(64, False, False), (1024, False, False),
                                              (1024, True, False), (512, True, True)])
def test_mixed_healpix_at_scale(nside, nest, tiled):
    from test_gpu_certified import _hp_engine
    Q1, dets, resp, gamma, _ = synth.workload(100, 30_000, seed=61, radius_deg=2.0, el=40.,
                                              throw=60., v_az=3.)
    Q2, _, _, _, _ = synth.workload(100, 30_000, seed=61, radius_deg=2.0, el=62., az0=0.,
                                    throw=60., v_az=3.)
    p, eng = _hp_engine(nside, nest, tiled)
    q = synth.native(p, np.concatenate([Q1, Q2]))
    _probe_hp(eng, q, dets, resp, tiled)


def test_mixed_healpix_edges():
    """The belt/cap boundary, phi = 0 and +-pi, and in-face edges of the
    equatorial belt (as in the certified tests)."""
    from test_gpu_certified import _hp_engine
    rng = np.random.default_rng(63)
    nside = 256
    n = 30000
    z_edge = rng.choice([2 / 3, -2 / 3], n // 3) + rng.choice([0., 1e-15, -1e-7, 1e-6], n // 3)
    lat_a, lon_a = np.arcsin(z_edge), rng.uniform(-np.pi, np.pi, n // 3)
    lat_b = rng.uniform(-1.1, 1.1, n // 3)
    lon_b = rng.choice([0., np.pi, -np.pi], n // 3) + rng.choice([0., 1e-9, -1e-7, 1e-6], n // 3)
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
        _probe_hp(eng, q, dets, resp, False)


@pytest.mark.parametrize("proj", ["TAN", "ZEA", "SIN"])
@pytest.mark.parametrize("tiled", [False, True])
def test_mixed_zenithal_at_scale(proj, tiled):
    Q, dets, resp, gamma, _ = synth.workload(100, 100_000, seed=65, radius_deg=1.0)
    p, eng = _engine((900, 1100), 0.25 * ARCMIN, tiled, proj=proj)
    q = synth.native(p, Q)
    res = _probe(eng, q, dets, resp, tiled)
    assert 0.2 < (res[0] > 0).mean() < 1.0


@pytest.mark.parametrize("proj", ["TAN", "ZEA", "SIN"])
def test_mixed_zenithal_edges(orc, proj):
    """Zenithal samples on pixel edges (and 1e-13 .. 1e-5 either side)."""
    from test_gpu_certified import _solve_lonlat
    rng = np.random.default_rng(67)
    p, eng = _engine((300, 400), 0.5 * ARCMIN, False, proj=proj)
    (ny, nx) = eng.naxis
    n = 20000
    ix = rng.integers(-2, nx + 2, n).astype(float)
    iy = rng.integers(-2, ny + 2, n).astype(float)
    jit = rng.choice([0., 1e-13, -1e-13, 1e-9, -1e-6, 1e-5, 0.5], n)
    gam = rng.uniform(0, np.pi, n)
    (dy, dx), (cry, crx) = eng.cdelt, eng.crpix
    u = (ix + jit - (crx - 0.5)) * abs(dx)
    v = (iy + jit - (cry - 0.5)) * dy
    lon, lat = _solve_lonlat(orc, eng, ix + jit, iy + jit, np.arctan2(u, v),
                             np.pi / 2 - np.hypot(u, v), gam)
    q = _quats_at(lon, lat, gam)
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    _probe(eng, q, dets, resp, False)


@pytest.mark.parametrize("proj", ["TAN", "ZEA", "SIN"])
def test_mixed_zenithal_whole_sky(proj):
    """Samples over the whole sphere on a wide zenithal map: the float32
    tier's guard sends the far side (and TAN's horizon) to the exact tiers
    and every pixel index stays equal."""
    rng = np.random.default_rng(69)
    p, eng = _engine((240, 240), 30 * ARCMIN, False, proj=proj)
    n = 40000
    lon = rng.uniform(-np.pi, np.pi, n)
    lat = np.arcsin(rng.uniform(-1, 1, n))
    q = _quats_at(lon, lat, rng.uniform(0, np.pi, n))
    dets = np.array([[1., 0., 0., 0.], [np.cos(0.3), 0., 0., np.sin(0.3)]])
    resp = np.array([[1., 1.], [0.7, 0.45]], np.float32)
    res = _probe(eng, q, dets, resp, False, pf_bound=PF_BOUND_GUARD)
    assert (res[0] > 0).mean() > 0.05
