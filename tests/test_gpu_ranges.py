"""Thread-assignment queries on the GPU: tile_hits, pixel_ranges and
tile_ranges against the oracle, and the coverage property of
test/test_proj_eng.py:103-151 (every on-map sample is assigned exactly
once; nearest-neighbour assignments have an empty serial bunch)."""
import numpy as np
import pytest

from helpers import Case, oracle_map

pytestmark = pytest.mark.gpu


def runs_from_labels(lab, n_domain):
    """The oracle's per-sample labels -> {(bunch, domain, det): [(a, b)]}."""
    out = {}
    n_det, n_time = lab.shape
    for d in range(n_det):
        row = lab[d]
        t = 0
        while t < n_time:
            e = t
            while e < n_time and row[e] == row[t]:
                e += 1
            if row[t] >= 0:
                key = (0, int(row[t]), d) if row[t] < n_domain else (1, 0, d)
                out.setdefault(key, []).append((t, e))
            t = e
    return out


def runs_from_ranges(R):
    out = {}
    for b, bunch in enumerate(R):
        for k, dom in enumerate(bunch):
            for d, r in enumerate(dom):
                iv = [tuple(x) for x in r.ranges().tolist()]
                if iv:
                    out[(b, k, d)] = iv
    return out


@pytest.mark.parametrize("tiled,bil", [(False, False), (False, True), (True, False),
                                       (True, True)])
def test_tile_hits_and_pixel_ranges(orc, gpulib, tiled, bil):
    c = Case(orc, coord="CAR", tiled=tiled, bilinear=bil, n_det=5, n_time=4000)
    if tiled:
        hits = np.array(c.eng.tile_hits(c.bore, c.dets))
        want = orc.tile_hits(c.pz, c.bore, c.dets, c.eng._n_tile())
        assert np.array_equal(hits, want)
    else:
        with pytest.raises(RuntimeError, match="No tiles"):
            c.eng.tile_hits(c.bore, c.dets)
    n = 3
    R = c.eng.pixel_ranges(c.bore, c.dets, None, n)
    lab = orc.labels(c.pz, c.bore, c.dets, 0, n)
    assert runs_from_ranges(R) == runs_from_labels(lab, n)


def test_tile_ranges(orc, gpulib):
    c = Case(orc, coord="CAR", tiled=True, n_det=5, n_time=4000)
    hits = np.array(c.eng.tile_hits(c.bore, c.dets))
    tiles = list(np.nonzero(hits)[0])
    groups = [tiles[0::2], tiles[1::2]]
    R = c.eng.tile_ranges(c.bore, c.dets, groups)
    td = np.full(c.eng._n_tile(), -1, np.int32)
    for i, g in enumerate(groups):
        td[g] = i
    lab = orc.labels(c.pz, c.bore, c.dets, 2, 2, tile_domain=td, n_tile=len(td))
    assert runs_from_ranges(R) == runs_from_labels(lab, 2)


def test_pixel_ranges_from_map(orc, gpulib):
    c = Case(orc, coord="CAR", ncomp=1, n_det=5, n_time=4000)
    tmap = np.zeros((1,) + c.eng._pix_shape())
    tmap[0, :, ::2] = 1.0   # alternate columns between threads 0 and 1
    R = c.eng.pixel_ranges(c.bore, c.dets, tmap, 2)
    flat, offs = oracle_map(tmap)
    lab = orc.labels(c.pz, c.bore, c.dets, 1, 2, dmap=(flat, offs))
    assert runs_from_ranges(R) == runs_from_labels(lab, 2)


@pytest.mark.parametrize("interpol", ["nearest", "bilinear"])
@pytest.mark.parametrize("method", ["simple", "domdir", "tiles"])
@pytest.mark.parametrize("tiled", [False, True])
def test_thread_coverage(orc, gpulib, interpol, method, tiled):
    from so3g_gb300.proj import Assembly, FocalPlane
    from so3g_gb300 import synth
    from so3g_gb300.proj import quat
    Q, dets, resp, gamma, sig = synth.workload(2, 3000, seed=3, rate=10., throw=3., v_az=2.)
    p = synth.car_projectionist((150, 200), 0.6 * np.pi / 180 / 60 * 10,
                                tile_shape=(50, 50) if tiled else None, interpol=interpol)
    if tiled:
        p.active_tiles = None
    asm = Assembly.attach(quat.G3VectorQuat(Q), FocalPlane(dets, resp))
    if method == "tiles" and not tiled:
        with pytest.raises(RuntimeError):
            p.assign_threads(asm, method=method, n_threads=3)
        return
    threads = p.assign_threads(asm, method=method, n_threads=3)
    assert isinstance(threads, list)
    counts0 = threads[0].mask().sum(axis=0)
    counts1 = np.zeros(counts0.shape, int)
    assert threads[0].shape == (3,) + sig.shape
    for t in threads[1:]:
        counts1 += t.mask().sum(axis=0)
    total = counts0 + counts1
    assert set(total.ravel()) <= {0, 1}
    pix = np.array(p.get_pixels(asm))
    if not tiled:
        on = pix[..., 0] >= 0
        if interpol == "nearest":
            assert np.array_equal(total == 1, on)
    if interpol == "nearest":
        assert counts1.sum() == 0
