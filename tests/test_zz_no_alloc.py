"""so3g_proj_to_map_noalloc, the to_map entry point for callers that cannot
allocate device memory (an application that owns all device memory through
its own pool or budget, or a binding that only passes buffers it holds).

Called through the C ABI, it must give the maps of so3g_proj_to_map within
the to_map tolerance of the other tests (1e-12 of the map's scale), on two
calls in a row -- the second with different tiles and segments, so nothing
of the first call's scratch may leak into it -- and must clear the error
record at each call.  It is also compared with the CPU oracle in every
pointing mode for a CAR, a TAN and a tiled HEALPix (NEST) map, and its
error record is read back after a call made without host_err.  This file
is collected last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12
ARCMIN = np.pi / 180 / 60


def _inputs(seed, tiled, n_det=6, n_time=20000):
    import torch
    from so3g_gb300 import synth
    Q, dets, resp, gamma, sig = synth.workload(n_det, n_time, seed=seed, rate=100., throw=5.)
    p = synth.car_projectionist((90, 140), 6 * ARCMIN, tile_shape=(32, 40) if tiled else None)
    q = synth.native(p, Q)
    eng = p.get_ProjEng("TQU")
    dev = torch.device("cuda", torch.cuda.current_device())
    t = dict(q=torch.from_numpy(q).to(dev), d=torch.from_numpy(dets).to(dev),
             r=torch.from_numpy(resp).to(dev), s=torch.from_numpy(sig).to(dev))
    return eng, t, n_det, n_time


def _tile_layout(eng, present):
    """Element offsets of the present tiles in one buffer; -1 = absent."""
    offs = np.full(eng._n_tile(), -1, dtype=np.int64)
    n = 0
    for i in range(eng._n_tile()):
        if i in present:
            offs[i] = n
            ty, tx = eng._tile_pix_shape(i)
            n += 3 * ty * tx
    return offs, n


def _segments(rng, n_det, n_time, k):
    seg = []
    for _ in range(k):
        d = int(rng.integers(0, n_det))
        a = int(rng.integers(0, n_time - 10))
        seg.append((d, a, int(min(n_time, a + rng.integers(1, 5000)))))
    return np.ascontiguousarray(np.array(seg, dtype=np.int32))


def _reference_call(lib, eng, t, n_det, n_time, seg, offs, size):
    """so3g_proj_to_map into a fresh buffer; returns (map, error record)."""
    import torch
    from so3g_gb300 import _abi
    assert lib.so3g_init() == 0
    dev = t["q"].device
    m = torch.zeros(max(size, 1), dtype=torch.float64, device=dev)
    ms = _abi.Map()
    ms.data = m.data_ptr()
    keep = []
    if offs is not None:
        to = torch.from_numpy(offs).to(dev)
        keep.append(to)
        ms.tile_offset = to.data_ptr()
        ms.n_tile = len(offs)
    rs = None
    if seg is not None:
        sd = torch.from_numpy(seg).to(dev)
        keep.append(sd)
        rs = _abi.Ranges()
        rs.seg = sd.data_ptr()
        rs.n_seg = len(seg)
        rs.max_len = int((seg[:, 2] - seg[:, 1]).max())
    err = torch.zeros(4, dtype=torch.int32, device=dev)
    rc = lib.so3g_proj_to_map(eng._pz(), t["q"].data_ptr(), n_time, t["d"].data_ptr(), n_det,
                              t["r"].data_ptr(), t["s"].data_ptr(), n_time, None, rs, ms,
                              _abi.ACCUM_WARP_RUNS, err.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _abi.last_error()
    torch.cuda.synchronize()
    return m.cpu().numpy(), err.cpu().numpy()


def _noalloc_call(lib, eng, t, n_det, n_time, seg, offs, size, accum):
    import torch
    from so3g_gb300 import _abi
    m = torch.zeros(max(size, 1), dtype=torch.float64, device=t["q"].device)
    host_err = np.full(4, -7, dtype=np.int32)
    rc = lib.so3g_proj_to_map_noalloc(
        eng._pz(), t["q"].data_ptr(), n_time, t["d"].data_ptr(), n_det, t["r"].data_ptr(),
        t["s"].data_ptr(), n_time, None,
        None if seg is None else seg.ctypes.data, 0 if seg is None else len(seg),
        m.data_ptr(), None if offs is None else offs.ctypes.data,
        0 if offs is None else len(offs), accum, host_err.ctypes.data,
        torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _abi.last_error()
    torch.cuda.synchronize()
    return m.cpu().numpy(), host_err


def _close(got, want):
    scale = max(np.abs(want).max(), 1e-300)
    assert np.abs(got - want).max() <= RTOL * scale


def test_noalloc_matches_to_map_twice():
    from so3g_gb300 import _abi
    lib = _abi.lib()
    rng = np.random.default_rng(11)
    # Call 1: tiled map with every tile, sample segments.
    eng, t, nd, nt = _inputs(1, tiled=True)
    offs, size = _tile_layout(eng, set(range(eng._n_tile())))
    seg = _segments(rng, nd, nt, 40)
    got, herr = _noalloc_call(lib, eng, t, nd, nt, seg, offs, size, _abi.ACCUM_WARP_RUNS)
    want, derr = _reference_call(lib, eng, t, nd, nt, seg, offs, size)
    assert np.all(herr == 0) and np.all(derr == 0)
    assert np.abs(want).max() > 0
    _close(got, want)
    # Call 2: other inputs, other segments, a different tile layout.
    eng2, t2, nd2, nt2 = _inputs(2, tiled=True)
    hits = np.array(eng2.tile_hits(t2["q"], t2["d"]))
    present = set(np.nonzero(hits)[0].tolist())
    offs2, size2 = _tile_layout(eng2, present)
    seg2 = _segments(rng, nd2, nt2, 25)
    got2, herr2 = _noalloc_call(lib, eng2, t2, nd2, nt2, seg2, offs2, size2, _abi.ACCUM_ATOMIC)
    want2, derr2 = _reference_call(lib, eng2, t2, nd2, nt2, seg2, offs2, size2)
    assert np.all(herr2 == 0) and np.all(derr2 == 0)
    _close(got2, want2)


def test_noalloc_untiled_all_samples_and_error_record():
    from so3g_gb300 import _abi
    lib = _abi.lib()
    eng, t, nd, nt = _inputs(3, tiled=False)
    size = 3 * eng.naxis[0] * eng.naxis[1]
    got, herr = _noalloc_call(lib, eng, t, nd, nt, None, None, size, _abi.ACCUM_WARP_RUNS)
    want, _ = _reference_call(lib, eng, t, nd, nt, None, None, size)
    assert np.all(herr == 0)
    _close(got, want)
    # A tiled call onto a missing tile sets the record; the next call clears it.
    eng2, t2, nd2, nt2 = _inputs(4, tiled=True)
    hits = np.array(eng2.tile_hits(t2["q"], t2["d"]))
    hit = np.nonzero(hits)[0]
    present = set(range(eng2._n_tile())) - {int(hit[0])}
    offs, size2 = _tile_layout(eng2, present)
    _, herr = _noalloc_call(lib, eng2, t2, nd2, nt2, None, offs, size2, _abi.ACCUM_WARP_RUNS)
    assert herr[0] == _abi.DEVERR_MISSING_TILE and 2**31 - 1 - herr[1] == hit[0]
    got, herr = _noalloc_call(lib, eng, t, nd, nt, None, None, size, _abi.ACCUM_WARP_RUNS)
    assert np.all(herr == 0)
    _close(got, want)


def test_noalloc_rejects_oversize():
    from so3g_gb300 import _abi
    lib = _abi.lib()
    eng, t, nd, nt = _inputs(5, tiled=False)
    seg = np.zeros((70000, 3), dtype=np.int32)
    rc = lib.so3g_proj_to_map_noalloc(eng._pz(), t["q"].data_ptr(), nt, t["d"].data_ptr(), nd,
                                      t["r"].data_ptr(), t["s"].data_ptr(), nt, None,
                                      seg.ctypes.data, len(seg), t["q"].data_ptr(), None, 0,
                                      _abi.ACCUM_ATOMIC, None, None)
    assert rc == -4
    assert "at most 65536 sample segments" in _abi.last_error()


def _noalloc_case(lib, c, mode, populate=None, seg=None):
    """so3g_proj_to_map_noalloc of a helpers.Case in pointing mode `mode`
    (tiled: the tiles in `populate`, or all); returns the flat map and its
    tile offsets (None if untiled)."""
    import torch
    from so3g_gb300 import _abi
    from helpers import oracle_map
    dev = torch.device("cuda", torch.cuda.current_device())
    flat, offs = oracle_map(c.blank((c.ncomp,), populate))
    m = torch.zeros(flat.size, dtype=torch.float64, device=dev)
    q, d, r, s = (torch.from_numpy(np.ascontiguousarray(x)).to(dev)
                  for x in (c.bore, c.dets, c.resp, c.signal))
    pz = c.eng._pz()
    pz.pointing = mode
    host_err = np.full(4, -7, dtype=np.int32)
    rc = lib.so3g_proj_to_map_noalloc(
        pz, q.data_ptr(), c.n_time, d.data_ptr(), c.n_det, r.data_ptr(), s.data_ptr(),
        c.n_time, None, None if seg is None else seg.ctypes.data,
        0 if seg is None else len(seg), m.data_ptr(),
        None if offs is None else offs.ctypes.data, 0 if offs is None else len(offs),
        _abi.ACCUM_WARP_RUNS, host_err.ctypes.data, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, _abi.last_error()
    assert np.all(host_err == 0)
    return m.cpu().numpy(), offs


@pytest.mark.parametrize("kind", ["CAR", "TAN", "HP_NEST_TILED"])
def test_noalloc_every_pointing_mode_against_oracle(orc, kind):
    """Each pointing mode twice in a row against the oracle (exact and
    certified: 1e-12 of the map's scale, the float64 summation order; mixed:
    float32 spin factors, 1e-6 of the scale) and against so3g_proj_to_map
    in the same mode (1e-12; mixed: within the mixed tolerance, as
    so3g_proj_to_map evaluates CAR pointing from its chunk models, the
    no-allocation entry point per sample)."""
    from so3g_gb300 import _abi
    from helpers import Case, oracle_map
    lib = _abi.lib()
    assert lib.so3g_init() == 0
    active = None
    if kind == "HP_NEST_TILED":
        c = Case(orc, coord="CAR", hp=(256, True, 8), tiled=True, n_det=6, n_time=6000,
                 seed=21)
        hits = np.array(c.eng.tile_hits(c.bore, c.dets))
        active = [int(i) for i in np.nonzero(hits)[0]]
        # The engine's own maps (to_map(None, ...)) hold the active tiles.
        c = Case(orc, coord="CAR", hp=(256, True, 8), tiled=True, n_det=6, n_time=6000,
                 seed=21, active=active)
    else:
        c = Case(orc, coord=kind, n_det=6, n_time=6000, seed=22)
    want, woffs = oracle_map(c.blank((c.ncomp,), active))
    orc.to_map(c.pz, c.bore, c.dets, c.resp, c.signal, None, want, woffs)
    scale = np.abs(want).max()
    assert scale > 0
    for mode, tol in ((_abi.POINTING_EXACT, 1e-12), (_abi.POINTING_CERTIFIED, 1e-12),
                      (_abi.POINTING_MIXED, 1e-6)):
        for _ in range(2):
            got, offs = _noalloc_case(lib, c, mode, active)
            assert offs is None or np.array_equal(offs, woffs)
            assert np.abs(got - want).max() <= tol * scale, (mode, np.abs(got - want).max())
        c.eng.pointing = mode
        ref = c.eng.to_map(None, c.bore, c.dets, c.resp, c.signal, None, None)
        from helpers import stack_map
        same = 1e-12 if mode != _abi.POINTING_MIXED else 2 * tol
        assert np.abs(got - stack_map(ref)).max() <= same * scale, mode


def test_noalloc_read_error_after_call_without_host_err():
    """A call onto an absent tile made with host_err = NULL leaves the
    record for so3g_noalloc_read_error; the next call clears it."""
    import torch
    from so3g_gb300 import _abi
    lib = _abi.lib()
    eng, t, nd, nt = _inputs(6, tiled=True)
    hits = np.array(eng.tile_hits(t["q"], t["d"]))
    hit = np.nonzero(hits)[0]
    offs, size = _tile_layout(eng, set(range(eng._n_tile())) - {int(hit[-1])})
    m = torch.zeros(max(size, 1), dtype=torch.float64, device=t["q"].device)
    stream = torch.cuda.current_stream().cuda_stream
    for want_err in (True, False):
        o = offs if want_err else _tile_layout(eng, set(range(eng._n_tile())))[0]
        if not want_err:
            m = torch.zeros(_tile_layout(eng, set(range(eng._n_tile())))[1],
                            dtype=torch.float64, device=t["q"].device)
        rc = lib.so3g_proj_to_map_noalloc(
            eng._pz(), t["q"].data_ptr(), nt, t["d"].data_ptr(), nd, t["r"].data_ptr(),
            t["s"].data_ptr(), nt, None, None, 0, m.data_ptr(), o.ctypes.data, len(o),
            _abi.ACCUM_ATOMIC, None, stream)
        assert rc == 0, _abi.last_error()
        rec = np.full(4, -7, dtype=np.int32)
        assert lib.so3g_noalloc_read_error(rec.ctypes.data, stream) == 0
        if want_err:
            assert rec[0] == _abi.DEVERR_MISSING_TILE and 2**31 - 1 - rec[1] == hit[-1]
        else:
            assert np.all(rec == 0)
    assert lib.so3g_noalloc_read_error(None, stream) == -1
