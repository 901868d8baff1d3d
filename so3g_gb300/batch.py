"""Many observations into one map: batched to_map / to_weight_map.

A map-maker accumulates many observations -- each with its own boresight,
focal plane, responses, signal and detector weights, of uneven length and
detector count -- into one map.  With the ProjEng interface that is one
``to_map`` call (one launch) per observation, as in the reference, where
each call is a ProjectionEngine::to_map (src/Projection.cxx:1924-1966).
``ObservationBatch`` instead describes all observations to the device once
(a table of ``so3g_obs`` records) and projects them with one persistent
launch: the work items (observation, detector, piece of ``piece`` samples)
of the whole batch are shared out over one wave of resident blocks.

* ``to_map`` / ``to_weight_map`` run one batched launch each (or, when
  the tuner finds it faster, one ordinary launch per observation).
* ``tune`` times a small grid of (piece, blocks) launch shapes on scratch
  maps and keeps the fastest; results are cached in a JSON file keyed by
  device, pixelization and batch size (``SO3G_GB300_TUNE_CACHE`` names the
  file; default ``~/.cache/so3g_gb300/tune.json``).
* ``graph`` captures the to_map (and optionally to_weight_map) launches in
  a CUDA graph, replayed with one call per map-making pass.

The sums equal those of one ``to_map`` call per observation, up to the
order of the float64 additions into the map.
"""
import ctypes
import json
import os
import time

import numpy as np
import torch

from . import _abi
from .projeng import (_ErrRecord, _MapArg, _device, _ensure_init, _stream, as_array,
                      DEFAULT_ACCUM)

# Launch shapes the tuner tries: samples per work item, and blocks per SM
# (0 = one persistent full wave, as many blocks as fit at once; -1 = one
# block per work item).  PER_OBSERVATION, as the blocks value, stands for
# one ordinary projection launch per observation instead of one batched
# launch; the tuner tries it once.
TUNE_PIECES = (2048, 4096, 8192, 16384, 32768)
TUNE_BLOCKS_PER_SM = (0, 2, 4, -1)
PER_OBSERVATION = -2
DEFAULT_PIECE = 8192


def _cache_path():
    p = os.environ.get("SO3G_GB300_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "so3g_gb300", "tune.json")


def _load_cache():
    try:
        with open(_cache_path()) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _store_cache(key, value):
    d = _load_cache()
    d[key] = value
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + ".%d.tmp" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


class Observation:
    """One observation: boresight (n_time, 4) and detector offsets
    (n_det, 4) float64 quaternions, response (n_det, 2) float32, signal
    (n_det, n_time) float32 (needed by to_map only) and optional
    det_weights (n_det,) float32.  Host arrays are copied to the device
    once, when the batch is built."""

    def __init__(self, boresight, dets, response, signal=None, det_weights=None):
        self.boresight = boresight
        self.dets = dets
        self.response = response
        self.signal = signal
        self.det_weights = det_weights


class ObservationBatch:
    """Observations projected together by ``eng`` (a ProjEng_* instance)."""

    def __init__(self, eng, observations):
        _ensure_init()
        dev = _device()
        self.eng = eng
        self._keep = []
        recs = (_abi.Obs * max(len(observations), 1))()
        self.n_obs = len(observations)
        self.n_samples = 0
        self.has_signal = True
        for i, ob in enumerate(observations):
            bore, dets, n_time, n_det, _ = eng._pointer(ob.boresight, ob.dets)
            resp = as_array(ob.response, "response", "float32", (n_det, 2))
            w = as_array(ob.det_weights, "det_weights", "float32", (n_det,), optional=True)
            sig = None
            if ob.signal is not None:
                sig = as_array(ob.signal, "signal", "float32", (n_det, n_time))
            bore, dets, resp, w = (None if a is None else _dev(a, dev)
                                   for a in (bore, dets, resp, w))
            r = recs[i]
            r.boresight = bore.data_ptr()
            r.dets = dets.data_ptr()
            r.response = resp.data_ptr()
            r.det_weights = w.data_ptr() if w is not None else None
            r.n_time = n_time
            r.n_det = n_det
            if sig is not None:
                sig = _dev_rows(sig, dev)
                r.signal = sig.data_ptr()
                r.sig_det_stride = sig.stride(0) if n_det > 1 else n_time
            else:
                r.signal = None
                r.sig_det_stride = 0
                if n_det * n_time:
                    self.has_signal = False
            self._keep.append((bore, dets, resp, w, sig))
            self.n_samples += n_det * n_time
        self._host_recs = recs
        raw = np.frombuffer(recs, dtype=np.uint8).copy()
        self._obs_dev = torch.from_numpy(raw).to(dev)
        self._plans = {}
        self._err = _ErrRecord()

    # -- plans ---------------------------------------------------------------------
    def plan(self, piece):
        """(device work_offset tensor, number of work items) for ``piece``."""
        if piece not in self._plans:
            off = np.zeros(self.n_obs + 1, dtype=np.int64)
            n_work = _abi.lib().so3g_batch_work_offsets(
                ctypes.cast(self._host_recs, ctypes.POINTER(_abi.Obs)), self.n_obs, piece,
                off.ctypes.data)
            if n_work < 0:
                raise ValueError("bad batch plan (piece %d)" % piece)
            self._plans[piece] = (torch.from_numpy(off).to(_device()), int(n_work))
        return self._plans[piece]

    def _launch(self, weight, m, piece, blocks, accum):
        acc = DEFAULT_ACCUM if accum is None else accum
        if blocks == PER_OBSERVATION:
            # One projection launch per observation (the piece is chosen by
            # the library); captured in a graph, they replay as one.
            lib, pz = _abi.lib(), self.eng._pz()
            for r, (bore, dets, resp, w, sig) in zip(self._host_recs, self._keep):
                if r.n_time == 0 or r.n_det == 0:
                    continue
                if weight:
                    rc = lib.so3g_proj_to_weight_map(
                        pz, r.boresight, r.n_time, r.dets, r.n_det, r.response, r.det_weights,
                        None, m.struct, acc, self._err.ptr, _stream())
                else:
                    rc = lib.so3g_proj_to_map(
                        pz, r.boresight, r.n_time, r.dets, r.n_det, r.response, r.signal,
                        r.sig_det_stride, r.det_weights, None, m.struct, acc, self._err.ptr,
                        _stream())
                _abi.check(rc, "to_weight_map" if weight else "to_map")
            return
        off, n_work = self.plan(piece)
        fn = (_abi.lib().so3g_proj_to_weight_map_batch if weight
              else _abi.lib().so3g_proj_to_map_batch)
        _abi.check(fn(self.eng._pz(), self._obs_dev.data_ptr(), self.n_obs, off.data_ptr(),
                      n_work, piece, blocks, m.struct,
                      DEFAULT_ACCUM if accum is None else accum, self._err.ptr, _stream()),
                   "to_weight_map batch" if weight else "to_map batch")

    def _shape(self, piece, blocks, weight):
        if piece is None or blocks is None:
            t = self.tuned(weight)
            if t is not None:
                piece = t[0] if piece is None else piece
                blocks = t[1] if blocks is None else blocks
        return (DEFAULT_PIECE if piece is None else int(piece),
                0 if blocks is None else int(blocks))

    # -- operators -----------------------------------------------------------------
    def to_map(self, map=None, piece=None, blocks=None, accum=None):
        """Adds every observation's signal into ``map`` (shape (n_comp,)
        + pixel shape, or a tile list); returns the map."""
        if not self.has_signal:
            raise ValueError("to_map needs a signal for every observation")
        eng = self.eng
        if map is None:
            map = eng.zeros(eng._ncomp, device=_device())
        m = _MapArg(eng, map, (eng._ncomp,)).upload()
        self._err.t.zero_()
        self._launch(False, m, *self._shape(piece, blocks, False), accum)
        self._err.raise_if_set()
        m.writeback()
        return map

    def to_weight_map(self, map=None, piece=None, blocks=None, accum=None):
        """Adds every observation's weights into ``map`` (shape (n_comp,
        n_comp) + pixel shape, or a tile list); returns the map."""
        eng = self.eng
        if map is None:
            map = eng.zeros((eng._ncomp, eng._ncomp), device=_device())
        m = _MapArg(eng, map, (eng._ncomp, eng._ncomp)).upload()
        self._err.t.zero_()
        self._launch(True, m, *self._shape(piece, blocks, True), accum)
        self._err.raise_if_set()
        m.writeback()
        return map

    # -- autotuning ----------------------------------------------------------------
    def _key(self, weight):
        pz = self.eng._pz()
        scale = int(np.log2(max(self.n_samples, 1)))
        return "%s|c%d|p%d|t%d|i%d|n%d|%s|obs%d|2^%d" % (
            torch.cuda.get_device_name(), pz.coord_sys, pz.pix_sys, pz.tiled, pz.interp,
            pz.n_comp, "w" if weight else "m", self.n_obs, scale)

    def tuned(self, weight=False):
        """Cached (piece, blocks) for this batch's kind, or None."""
        v = _load_cache().get(self._key(weight))
        if isinstance(v, dict) and "piece" in v and "blocks" in v:
            return int(v["piece"]), int(v["blocks"])
        return None

    def tune(self, weight=False, pieces=TUNE_PIECES, blocks_per_sm=TUNE_BLOCKS_PER_SM,
             reps=2, store=True, per_observation=True):
        """Times every (piece, blocks) candidate on a scratch map (after
        one warm-up launch), and one launch per observation when
        ``per_observation``; returns the fastest as (piece, blocks) and
        stores it in the cache when ``store``.  The timings are in
        ``self.tune_log``."""
        eng = self.eng
        lead = (eng._ncomp, eng._ncomp) if weight else (eng._ncomp,)
        m = _MapArg(eng, eng.zeros(lead, device=_device()), lead).upload()
        sms = torch.cuda.get_device_properties(_device()).multi_processor_count
        stream = torch.cuda.current_stream()
        log = []
        self._launch(weight, m, pieces[0], max(blocks_per_sm[0], 0) * sms, None)
        shapes = [(piece, bps * sms if bps >= 0 else -1) for piece in pieces
                  for bps in blocks_per_sm]
        if per_observation:
            shapes.append((DEFAULT_PIECE, PER_OBSERVATION))
        for piece, blocks in shapes:
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(reps):
                self._launch(weight, m, piece, blocks, None)
            t1.record(stream)
            t1.synchronize()
            log.append({"piece": piece, "blocks": blocks, "ms": t0.elapsed_time(t1) / reps})
        self._err.t.zero_()
        best = min(log, key=lambda r: r["ms"])
        self.tune_log = log
        if store:
            _store_cache(self._key(weight), {"piece": best["piece"], "blocks": best["blocks"],
                                             "ms": best["ms"], "when": time.time()})
        return best["piece"], best["blocks"]

    # -- CUDA graphs ---------------------------------------------------------------
    def graph(self, map, weight_map=None, accum=None, map_shape=None, weight_shape=None):
        """Captures to_map into ``map`` (and to_weight_map into
        ``weight_map``) as one CUDA graph; returns a BatchGraph.  Both maps
        must be CUDA tensors (or lists of CUDA tiles) that stay alive and
        in place while the graph is used.  ``map_shape`` / ``weight_shape``
        are (piece, blocks) launch shapes; by default the tuned ones."""
        return BatchGraph(self, map, weight_map, accum, map_shape, weight_shape)


class BatchGraph:
    """A captured batched projection.  ``replay()`` adds the batch into the
    captured maps again; ``check()`` raises if a launch recorded a device
    error (a missing tile or a pixel out of range)."""

    def __init__(self, batch, map, weight_map, accum, map_shape=None, weight_shape=None):
        eng = batch.eng
        if not batch.has_signal:
            raise ValueError("to_map needs a signal for every observation")
        self.batch = batch
        self._maps = []
        ops = [(False, map, (eng._ncomp,))]
        if weight_map is not None:
            ops.append((True, weight_map, (eng._ncomp, eng._ncomp)))
        launches = []
        for weight, obj, lead in ops:
            m = _MapArg(eng, obj, lead, name="weight_map" if weight else "map")
            m.upload()
            if m.host is not None or m._host_tiles is not None:
                raise TypeError("graph capture needs maps resident on the device "
                                "(CUDA tensors)")
            shape = (weight_shape if weight else map_shape) or (None, None)
            piece, blocks = batch._shape(shape[0], shape[1], weight)
            batch.plan(piece)
            launches.append((weight, m, piece, blocks))
            self._maps.append(m)
        batch._err.t.zero_()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        n0 = _abi.lib().so3g_launch_count()
        with torch.cuda.graph(self.graph):
            for weight, m, piece, blocks in launches:
                batch._launch(weight, m, piece, blocks, accum)
        # Kernel launches recorded in the graph (each replay runs them all).
        self.launches = int(_abi.lib().so3g_launch_count() - n0)

    def replay(self):
        self.graph.replay()

    def check(self):
        self.batch._err.raise_if_set()


def _dev(a, dev):
    if isinstance(a, torch.Tensor):
        return a.contiguous() if a.is_cuda else a.contiguous().to(dev)
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _dev_rows(sig, dev):
    """Signal on the device with unit stride along time (rows may be
    strided)."""
    if isinstance(sig, torch.Tensor) and sig.is_cuda:
        if sig.dim() == 2 and sig.stride(1) == 1 and sig.stride(0) >= sig.shape[1]:
            return sig
        return sig.contiguous()
    return _dev(sig, dev)


__all__ = ["Observation", "ObservationBatch", "BatchGraph"]
