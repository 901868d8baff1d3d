"""CPU oracle for the so3g ProjectionEngine hot path -- TEST INFRASTRUCTURE.

A ctypes wrapper around oracle/proj_oracle.cpp, the operation-by-operation
restatement of the reference arithmetic (so3g src/Projection.cxx,
include/so_linterp.h, src/healpix_bare.c).  Only the tests, the smoke
check of __graft_entry__ and the CPU-baseline leg of bench.py use it, to
check results or as the timed CPU baseline; the so3g_gb300 package never
does.

Parity pin: the oracle's trig tables and HEALPix ang2pix are checked
against golden vectors generated from the reference's own so_linterp.h and
healpix_bare.c (tests/golden/), its pointing/projection against the
reference's analytic known-answer tests (tests/test_oracle_kat.py), and
every engine method against the reference's own ProjectionEngine compiled
from src/Projection.cxx with stand-in boost.python/spt3g headers
(oracle/ref_engine.cpp, tests/test_oracle_reference.py): bit for bit.
The last bit of boost's quaternion product is not pinned (boost is not
installed; both sum each component left to right).
"""
import ctypes

import numpy as np

from . import build as _build

_V = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64


class Sched(ctypes.Structure):
    """orc_sched of proj_oracle.h."""
    _fields_ = [("seg", _V), ("n_seg", _I32), ("n_thread", _I32),
                ("thread_offset", _V), ("n_bunch", _I32), ("_pad", _I32),
                ("bunch_offset", _V)]


def _p(a):
    return None if a is None else a.ctypes.data


def schedule(thread_intervals, n_det):
    """Restates derive_ranges (src/Projection.cxx:1856-1922): nested
    [bunch][thread][det] Ranges -> (seg, thread_offset, bunch_offset)."""
    ti = thread_intervals

    def is_r(x):
        return hasattr(x, "ranges") and hasattr(x, "count")

    if is_r(ti[0]):
        bunches = [[list(ti)]]
    elif is_r(ti[0][0]):
        bunches = [[list(x) for x in ti]]
    else:
        bunches = [[list(y) for y in x] for x in ti]
    seg, toff, boff = [], [0], [0]
    for bunch in bunches:
        for thread in bunch:
            assert len(thread) == n_det
            for det, r in enumerate(thread):
                for a, b in np.asarray(r.ranges()).reshape(-1, 2):
                    seg.append((det, a, b))
            toff.append(len(seg))
        boff.append(len(toff) - 1)
    return (np.asarray(seg, dtype=np.int32).reshape(-1, 3),
            np.asarray(toff, dtype=np.int32), np.asarray(boff, dtype=np.int32))


class Schedule:
    """A thread_intervals argument converted once (Oracle.schedule) for
    repeated projections."""

    def __init__(self, s, keep):
        self.s = s
        self.keep = keep


class Oracle:
    def schedule(self, threads, n_det):
        """thread_intervals -> Schedule, accepted wherever `threads` is."""
        s, keep = self._sched(threads, n_det)
        return Schedule(s, keep)

    def __init__(self, threads=None):
        self.lib = ctypes.CDLL(_build.build_oracle())
        L = self.lib
        for name in ("orc_init", "orc_set_threads"):
            getattr(L, name).restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_get_tables.argtypes = [_V, _V, _I32]
        L.orc_asin.restype = ctypes.c_double
        L.orc_asin.argtypes = [ctypes.c_double]
        L.orc_atan2.restype = ctypes.c_double
        L.orc_atan2.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_ang2pix.restype = _I64
        L.orc_ang2pix.argtypes = [_I64, _I32, ctypes.c_double, ctypes.c_double]
        L.orc_last_error.restype = ctypes.c_char_p
        from so3g_gb300._abi import Map, Pixelization, PrecompGeom
        P, PM, PS, PG = (ctypes.POINTER(Pixelization), ctypes.POINTER(Map),
                         ctypes.POINTER(Sched), ctypes.POINTER(PrecompGeom))
        sigs = {
            "orc_coords": [P, _V, _I32, _V, _I32, _V],
            "orc_pixels": [P, _V, _I32, _V, _I32, _V],
            "orc_pointing_matrix": [P, _V, _I32, _V, _I32, _V, _V, _V],
            "orc_tile_hits": [P, _V, _I32, _V, _I32, _V, _I32],
            "orc_domain_labels": [P, _V, _I32, _V, _I32, _I32, _I32, PM, _V, _I32, _V],
            "orc_to_map": [P, _V, _I32, _V, _I32, _V, _V, _I64, _V, PS, PM, _V],
            "orc_to_weight_map": [P, _V, _I32, _V, _I32, _V, _V, PS, PM, _V],
            "orc_from_map": [P, _V, _I32, _V, _I32, _V, PM, _V, _I64, _V],
            "orc_precomp_to_map": [PG, _V, _V, _I32, _I32, _V, _I64, _V, PS, PM, _V],
            "orc_precomp_to_weight_map": [PG, _V, _V, _I32, _I32, _V, PS, PM, _V],
            "orc_precomp_from_map": [PG, _V, _V, _I32, _I32, PM, _V, _I64, _V],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.restype = ctypes.c_int
            fn.argtypes = args
        L.orc_init()
        if threads is not None:
            L.orc_set_threads(int(threads))

    def set_threads(self, n):
        return self.lib.orc_set_threads(int(n))

    def _check(self, rc):
        if rc != 0:
            raise ValueError(self.lib.orc_last_error().decode())

    # -- scalars -------------------------------------------------------------
    def tables(self):
        a = np.empty(1 << 14)
        b = np.empty(1 << 14)
        self._check(self.lib.orc_get_tables(_p(a), _p(b), 1 << 14))
        return a, b

    def asin(self, x):
        return self.lib.orc_asin(float(x))

    def atan2(self, y, x):
        return self.lib.orc_atan2(float(y), float(x))

    def ang2pix(self, nside, nest, theta, phi):
        return self.lib.orc_ang2pix(int(nside), int(nest), float(theta), float(phi))

    # -- pointing ------------------------------------------------------------
    @staticmethod
    def _in(bore, dets):
        bore = np.ascontiguousarray(bore, dtype=np.float64)
        dets = np.ascontiguousarray(dets, dtype=np.float64)
        return bore, dets, len(bore), len(dets)

    def coords(self, pz, bore, dets):
        bore, dets, nt, nd = self._in(bore, dets)
        out = np.zeros((nd, nt, 4))
        self._check(self.lib.orc_coords(ctypes.byref(pz), _p(bore), nt, _p(dets), nd, _p(out)))
        return out

    @staticmethod
    def _check_index_count(pz, index_count):
        """Pixel index entries per sample: 1 (+1 tiled) for HEALPix, 2 (+1
        tiled) for flat maps; the C side writes that many."""
        want = (1 if pz.pix_sys == 1 else 2) + (1 if pz.tiled else 0)
        if index_count != want:
            raise ValueError("index_count %d; this pixelization has %d" % (index_count, want))

    def pixels(self, pz, bore, dets, index_count):
        self._check_index_count(pz, index_count)
        bore, dets, nt, nd = self._in(bore, dets)
        out = np.zeros((nd, nt, index_count), dtype=np.int32)
        self._check(self.lib.orc_pixels(ctypes.byref(pz), _p(bore), nt, _p(dets), nd, _p(out)))
        return out

    def pointing_matrix(self, pz, bore, dets, resp, index_count):
        self._check_index_count(pz, index_count)
        bore, dets, nt, nd = self._in(bore, dets)
        resp = np.ascontiguousarray(resp, dtype=np.float32)
        pix = np.zeros((nd, nt, index_count), dtype=np.int32)
        proj = np.zeros((nd, nt, pz.n_comp), dtype=np.float32)
        self._check(self.lib.orc_pointing_matrix(ctypes.byref(pz), _p(bore), nt, _p(dets), nd,
                                                 _p(resp), _p(pix), _p(proj)))
        return pix, proj

    def tile_hits(self, pz, bore, dets, n_tile):
        bore, dets, nt, nd = self._in(bore, dets)
        hits = np.zeros(n_tile, dtype=np.int64)
        self._check(self.lib.orc_tile_hits(ctypes.byref(pz), _p(bore), nt, _p(dets), nd,
                                           _p(hits), n_tile))
        return hits

    def labels(self, pz, bore, dets, mode, n_domain, dmap=None, tile_domain=None, n_tile=0):
        """Per-sample domain labels; dmap = (flat float64 data, tile offsets
        or None)."""
        bore, dets, nt, nd = self._in(bore, dets)
        lab = np.zeros((nd, nt), dtype=np.int32)
        ms = None
        keep = []
        if dmap is not None:
            from so3g_gb300._abi import Map
            data, offs = dmap
            ms = Map()
            ms.data = _p(data)
            ms.tile_offset = _p(offs)
            ms.n_tile = 0 if offs is None else len(offs)
            keep.append(ms)
        td = None if tile_domain is None else np.ascontiguousarray(tile_domain, dtype=np.int32)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_domain_labels(
            ctypes.byref(pz), _p(bore), nt, _p(dets), nd, int(mode), int(n_domain),
            ctypes.byref(ms) if ms is not None else None, _p(td), int(n_tile), _p(lab)))
        return lab

    # -- projection ----------------------------------------------------------
    @staticmethod
    def _map(data, offsets):
        from so3g_gb300._abi import Map
        m = Map()
        m.data = _p(data)
        m.tile_offset = _p(offsets)
        m.n_tile = 0 if offsets is None else len(offsets)
        return m

    @staticmethod
    def _sched(threads, n_det):
        if threads is None:
            return None, None
        if isinstance(threads, Schedule):
            return threads.s, threads.keep
        seg, toff, boff = schedule(threads, n_det)
        s = Sched()
        s.seg = _p(seg)
        s.n_seg = len(seg)
        s.thread_offset = _p(toff)
        s.n_thread = len(toff) - 1
        s.bunch_offset = _p(boff)
        s.n_bunch = len(boff) - 1
        return s, (seg, toff, boff)

    def to_map(self, pz, bore, dets, resp, signal, det_weights, map_data, tile_offset=None,
               threads=None):
        bore, dets, nt, nd = self._in(bore, dets)
        resp = np.ascontiguousarray(resp, dtype=np.float32)
        sig = np.ascontiguousarray(signal, dtype=np.float32)
        w = None if det_weights is None else np.ascontiguousarray(det_weights, np.float32)
        s, keep = self._sched(threads, nd)
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_to_map(
            ctypes.byref(pz), _p(bore), nt, _p(dets), nd, _p(resp), _p(sig),
            _I64(sig.shape[1] if sig.ndim == 2 else nt), _p(w),
            ctypes.byref(s) if s is not None else None, ctypes.byref(m), _p(err)))
        return err

    def to_weight_map(self, pz, bore, dets, resp, det_weights, map_data, tile_offset=None,
                      threads=None):
        bore, dets, nt, nd = self._in(bore, dets)
        resp = np.ascontiguousarray(resp, dtype=np.float32)
        w = None if det_weights is None else np.ascontiguousarray(det_weights, np.float32)
        s, keep = self._sched(threads, nd)
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_to_weight_map(
            ctypes.byref(pz), _p(bore), nt, _p(dets), nd, _p(resp), _p(w),
            ctypes.byref(s) if s is not None else None, ctypes.byref(m), _p(err)))
        return err

    def from_map(self, pz, bore, dets, resp, map_data, signal, tile_offset=None):
        """Accumulates into `signal` (float32 (n_det, n_time), contiguous)."""
        bore, dets, nt, nd = self._in(bore, dets)
        resp = np.ascontiguousarray(resp, dtype=np.float32)
        assert signal.dtype == np.float32 and signal.flags.c_contiguous
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_from_map(
            ctypes.byref(pz), _p(bore), nt, _p(dets), nd, _p(resp), ctypes.byref(m),
            _p(signal), _I64(signal.shape[1]), _p(err)))
        return err

    # -- precomputed pointing ------------------------------------------------
    @staticmethod
    def _geom(n_comp, naxis=None, tile_dims=None):
        from so3g_gb300._abi import PrecompGeom
        g = PrecompGeom()
        g.n_comp = n_comp
        if tile_dims is not None:
            g.tiled = 1
            g.tile_dims = _p(tile_dims)
        else:
            g.naxis[0], g.naxis[1] = naxis
        return g

    def precomp_to_map(self, pixel, spin, signal, det_weights, map_data, naxis=None,
                       tile_offset=None, tile_dims=None, threads=None):
        pixel = np.ascontiguousarray(pixel, np.int32)
        spin = np.ascontiguousarray(spin, np.float32)
        sig = np.ascontiguousarray(signal, np.float32)
        nd, nt = pixel.shape[:2]
        g = self._geom(spin.shape[2], naxis, tile_dims)
        w = None if det_weights is None else np.ascontiguousarray(det_weights, np.float32)
        s, keep = self._sched(threads, nd)
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_precomp_to_map(
            ctypes.byref(g), _p(pixel), _p(spin), nd, nt, _p(sig), _I64(nt), _p(w),
            ctypes.byref(s) if s is not None else None, ctypes.byref(m), _p(err)))
        return err

    def precomp_to_weight_map(self, pixel, spin, det_weights, map_data, naxis=None,
                              tile_offset=None, tile_dims=None, threads=None):
        pixel = np.ascontiguousarray(pixel, np.int32)
        spin = np.ascontiguousarray(spin, np.float32)
        nd, nt = pixel.shape[:2]
        g = self._geom(spin.shape[2], naxis, tile_dims)
        w = None if det_weights is None else np.ascontiguousarray(det_weights, np.float32)
        s, keep = self._sched(threads, nd)
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_precomp_to_weight_map(
            ctypes.byref(g), _p(pixel), _p(spin), nd, nt, _p(w),
            ctypes.byref(s) if s is not None else None, ctypes.byref(m), _p(err)))
        return err

    def precomp_from_map(self, pixel, spin, map_data, signal, naxis=None, tile_offset=None,
                         tile_dims=None):
        pixel = np.ascontiguousarray(pixel, np.int32)
        spin = np.ascontiguousarray(spin, np.float32)
        nd, nt = pixel.shape[:2]
        assert signal.dtype == np.float32 and signal.flags.c_contiguous
        g = self._geom(spin.shape[2], naxis, tile_dims)
        m = self._map(map_data, tile_offset)
        err = np.zeros(4, dtype=np.int32)
        self._check(self.lib.orc_precomp_from_map(
            ctypes.byref(g), _p(pixel), _p(spin), nd, nt, ctypes.byref(m), _p(signal),
            _I64(nt), _p(err)))
        return err


def pack_tiles(tiles):
    """List of tile arrays (None = absent) -> (flat float64 buffer, int64
    element offsets with -1 for absent tiles)."""
    offs = np.full(len(tiles), -1, dtype=np.int64)
    parts = []
    n = 0
    for i, t in enumerate(tiles):
        if t is None:
            continue
        offs[i] = n
        parts.append(np.ascontiguousarray(t, dtype=np.float64).ravel())
        n += parts[-1].size
    flat = np.concatenate(parts) if parts else np.zeros(1)
    return flat, offs


def unpack_tiles(flat, offs, like):
    out = []
    for i, t in enumerate(like):
        if t is None or offs[i] < 0:
            out.append(None)
        else:
            out.append(flat[offs[i]:offs[i] + t.size].reshape(t.shape))
    return out
