"""ProjEng_* classes: the drop-in for so3g's ProjectionEngine bindings.

so3g exposes one Python class per template instance of ProjectionEngine
(src/Projection.cxx:2258-2358): ``ProjEng_<C>_<S>_<T>[_Bilinear]`` for the
coordinate systems C in Flat, Quat, CAR, CEA, ARC, SIN, TAN, ZEA, spins S in
T, QU, TQU and tilings T in NonTiled, Tiled; ``ProjEng_HP_<S>_<T>`` for
HEALPix; and ``ProjEng_Precomp_<T>``.  This module builds the same class
family over the GB300 CUDA library.  Constructor arguments, method names,
argument order and meaning, return values, in-place mutation of ``map`` and
``signal`` and the exception classes and messages follow the reference.

Arguments may be numpy arrays (or other buffer-protocol objects), CPU torch
tensors or CUDA torch tensors.  Host arguments are copied to the current
CUDA device, the kernels run, and outputs are copied back into the caller's
arrays before the call returns; a large host signal that the device can
reach in place (page-locked, or pageable on a host with coherent device
access) is instead read and written by the kernels where it lies, and one
that it cannot is streamed through the device in chunks.  CUDA tensors are used in place on the
current stream (no copies); outputs created by the call are then CUDA
tensors too.  Every call runs the CUDA kernels: there is no CPU path.
"""
import ctypes
import gc
import os

import weakref

import numpy as np
import torch

from . import _abi
from .ranges import RangesInt32

INT32_MAX = 2**31 - 1

# Default scatter accumulator: warp pre-reduction of pixel runs.
DEFAULT_ACCUM = _abi.ACCUM_WARP_RUNS
# Default pointing evaluation: certified double-float where available (its
# results equal the exact float64 path's).  An engine's ``pointing``
# attribute selects another: _abi.POINTING_EXACT (float64 everywhere) or
# _abi.POINTING_MIXED (float32 pointing with certified pixel indices; maps
# within ~1e-7 of the float64 path's).
DEFAULT_POINTING = _abi.POINTING_CERTIFIED


# ---------------------------------------------------------------------------
# Exceptions (include/exceptions.h:42-116; numpy_assist.h:141-234).

def _shape_string(shape):
    parts = []
    for s in shape:
        parts.append("*" if s == -1 else "..." if s == -2 else str(s))
    return "(" + ", ".join(parts) + ")"


def buffer_error(name):
    return TypeError("Argument '%s' does not expose buffer protocol, is not contiguous, "
                     "or does not export a format." % name)


def dtype_error(name, tname):
    return ValueError("Expected buffer '%s' to contain items of type %s." % (name, tname))


def shape_error(name, detail):
    return RuntimeError("Buffer '%s' has incompatible shape: %s." % (name, detail))


def tiling_error(idx, msg):
    return RuntimeError("Tiling problem (index %d): %s" % (idx, msg))


# ---------------------------------------------------------------------------
# Device plumbing.

_NP = {"float64": np.dtype(np.float64), "float32": np.dtype(np.float32),
       "int32": np.dtype(np.int32)}
_TORCH = {"float64": torch.float64, "float32": torch.float32, "int32": torch.int32}
_initialized = set()


def _device():
    if not torch.cuda.is_available():
        raise _abi.LibraryError("so3g_gb300 needs a CUDA device (none is visible)")
    return torch.device("cuda", torch.cuda.current_device())


def _ensure_init():
    dev = _device()
    if dev.index not in _initialized:
        _abi.check(_abi.lib().so3g_init(), "so3g_init")
        _initialized.add(dev.index)
    return dev


def _stream():
    return torch.cuda.current_stream().cuda_stream


def _is_cuda(x):
    return isinstance(x, torch.Tensor) and x.is_cuda


def _match_shape(name, pattern, shape):
    """BufferWrapper shape match: -1 matches one axis, -2 any number."""
    i = j = 0
    pattern = list(pattern)
    while i < len(pattern):
        if pattern[i] == -2:
            j = len(shape) - (len(pattern) - i) + 1
        elif j >= len(shape):
            break
        elif pattern[i] == -1 or pattern[i] == shape[j]:
            j += 1
        else:
            break
        i += 1
    if i != len(pattern) or j != len(shape):
        # numpy_assist.h:201-206 ends the detail with its own period, to
        # which the shape_exception message adds another.
        raise shape_error(name, "Expected %s but got %s." % (_shape_string(pattern),
                                                            _shape_string(shape)))


def as_array(obj, name, tname, shape=None, optional=False):
    """Validate a buffer argument; returns an ndarray or a torch tensor."""
    if obj is None:
        if optional:
            return None
        raise buffer_error(name)
    if isinstance(obj, torch.Tensor):
        if obj.dtype != _TORCH[tname]:
            raise dtype_error(name, tname)
        arr = obj
    else:
        if not isinstance(obj, np.ndarray):
            try:
                obj = np.asarray(memoryview(obj))
            except TypeError:
                raise buffer_error(name) from None
        if obj.dtype.newbyteorder("=") != _NP[tname] or obj.dtype.kind != _NP[tname].kind:
            raise dtype_error(name, tname)
        arr = obj
    if shape is not None:
        _match_shape(name, shape, tuple(arr.shape))
    return arr


def to_device(x, tname):
    """Contiguous CUDA tensor holding x (a no-op for a contiguous CUDA tensor)."""
    dev = _device()
    if isinstance(x, torch.Tensor):
        if x.is_cuda:
            return x.contiguous()
        return x.contiguous().to(dev, non_blocking=x.is_pinned())
    a = np.ascontiguousarray(x, dtype=_NP[tname])
    if not a.flags.writeable:
        a = a.copy()
    return torch.from_numpy(a).to(dev)


def copy_back(host, dev):
    """Copy a device result into a host array / tensor in place."""
    if isinstance(host, torch.Tensor):
        if host.is_cuda:
            if host.data_ptr() != dev.data_ptr():
                host.copy_(dev.view(host.shape))
            return
        host.copy_(dev.view(host.shape))
        return
    if host.flags.c_contiguous and host.flags.writeable:
        torch.from_numpy(host).copy_(dev.view(host.shape))
    else:
        host[...] = dev.cpu().numpy().reshape(host.shape)


def _ptr(t):
    return None if t is None else t.data_ptr()


class _ErrRecord:
    """The 4 x int32 device error record of a projection call."""

    def __init__(self):
        self.t = torch.zeros(4, dtype=torch.int32, device=_device())

    @property
    def ptr(self):
        return self.t.data_ptr()

    def raise_if_set(self):
        code, a, b, c = (int(v) for v in self.t.cpu())
        if code == _abi.DEVERR_MISSING_TILE:
            raise tiling_error(INT32_MAX - a,
                               "Attempted pointing operation on non-instantiated tile.")
        if code == _abi.DEVERR_PIXEL_RANGE:
            raise ValueError("Pixel index out of range for map/tile %d (detector %d, "
                             "sample %d)." % (a, b, c))
        if code != 0:
            raise RuntimeError("device error record %d" % code)


# ---------------------------------------------------------------------------
# Signal-like arguments (SignalSpace<T>, src/Projection.cxx:1212-1298).

class _Signal:
    """A (n_det, n_time[, k]) argument given as a 2/3-d array, a list of
    per-detector arrays, a torch tensor or None.  The constructor only
    validates (like SignalSpace); upload() moves the data to the device."""

    def __init__(self, obj, name, tname, dims, create, device_mode):
        self.name, self.tname = name, tname
        self.device_mode = device_mode
        self.obj = obj
        self.rows = None      # list of row arrays (list input), written back
        self.host = None      # host array / tensor written back
        self.dev = None
        self._src = None      # what upload() copies
        dims = list(dims)
        if obj is None:
            if not create:
                raise buffer_error(name)
            if any(d < 0 for d in dims):
                raise shape_error(name, "Cannot create space with wildcard dimensons.")
            self.dims = dims
            self._create = True
            return
        self._create = False
        if isinstance(obj, torch.Tensor):
            arr = as_array(obj, name, tname)
            self._check_dims(dims, tuple(arr.shape), len(arr))
            self._src = arr
            self.ret = arr
            return
        if isinstance(obj, (list, tuple)):
            items = [as_array(x, name, tname) for x in obj]
            if dims[0] == -1:
                dims[0] = len(items)
                if dims[0] == 0:
                    raise shape_error(name, "has not been tested on shape 0 objects")
            elif len(items) != dims[0]:
                raise shape_error(name, "must contain (n_det) vectors")
            sub = dims[1:]
            for i, it in enumerate(items):
                _match_shape(name, sub, tuple(it.shape))
                if i == 0:
                    sub = list(it.shape)
            self.dims = [dims[0]] + sub
            self.rows = items
            self.ret = obj if isinstance(obj, list) else list(obj)
            return
        # Any other buffer: listified by its first axis.
        arr = as_array(obj, name, tname)
        self._check_dims(dims, tuple(arr.shape), len(arr))
        self._src = arr
        self.host = arr
        self.ret = list(arr)

    def _check_dims(self, dims, shape, n):
        if dims[0] == -1:
            dims[0] = n
            if n == 0:
                raise shape_error(self.name, "has not been tested on shape 0 objects")
        elif n != dims[0]:
            raise shape_error(self.name, "must contain (n_det) vectors")
        _match_shape(self.name, dims[1:], shape[1:])
        self.dims = [dims[0]] + list(shape[1:])

    def upload(self):
        tname = self.tname
        if self._create:
            shape = tuple(self.dims)
            self.dev = torch.zeros(shape, dtype=_TORCH[tname], device=_device())
            if self.device_mode:
                self.ret = self.dev
            else:
                self.host = np.zeros(shape, dtype=_NP[tname])
                self.ret = list(self.host)
        elif self.rows is not None:
            items = self.rows
            if any(isinstance(x, torch.Tensor) for x in items):
                stacked = torch.stack([x if isinstance(x, torch.Tensor) else
                                       torch.from_numpy(np.asarray(x)) for x in items])
                self.dev = to_device(stacked, tname)
            else:
                self.dev = to_device(np.stack(items), tname)
        else:
            arr = self._src
            if _is_cuda(arr) and arr.dim() >= 2 and arr.stride(-1) == 1 and (
                    arr.dim() == 2 or arr.is_contiguous()):
                self.dev = arr
            else:
                self.dev = to_device(arr, tname)
                self.host = arr
        return self

    @property
    def det_stride(self):
        return self.dev.stride(0)

    def writeback(self):
        if self.rows is not None:
            for i, r in enumerate(self.rows):
                copy_back(r, self.dev[i])
        elif self.host is not None:
            copy_back(self.host, self.dev)


# ---------------------------------------------------------------------------
# Thread intervals (derive_ranges, src/Projection.cxx:1856-1922).

from .ranges import DeviceRangesMatrix  # noqa: E402


def _is_ranges(x):
    return isinstance(x, RangesInt32)


def derive_ranges(thread_intervals, n_det, n_time, arg_name="thread_intervals"):
    """Returns [bunch][thread][det] lists of RangesInt32, or None for 'all
    samples in one thread'."""
    ti = thread_intervals
    if ti is None:
        return None
    if _is_ranges(ti[0]):
        bunches = [[list(ti)]]
    elif _is_ranges(ti[0][0]):
        bunches = [[list(x) for x in ti]]
    elif _is_ranges(ti[0][0][0]):
        bunches = [[list(y) for y in x] for x in ti]
    else:
        raise TypeError("%s: expected Ranges, a RangesMatrix or a list of them" % arg_name)
    for bunch in bunches:
        for ival in bunch:
            if len(ival) != n_det:
                raise shape_error(arg_name, "Expected RangesMatrix with n_det=%d but "
                                  "encountered n_det=%d" % (n_det, len(ival)))
            for r in ival:
                if r.count != n_time:
                    raise shape_error(arg_name, "Expected RangesMatrix with n_time=%d but "
                                      "encountered n_time=%d" % (n_time, r.count))
    return bunches


def flatten_ranges(bunches):
    """(det, start, end) segments in the reference's processing order, plus
    thread and bunch offsets."""
    segs, toff, boff = [], [0], [0]
    count = 0
    for bunch in bunches:
        for ival in bunch:
            for det, r in enumerate(ival):
                rr = r.ranges()
                if len(rr):
                    s = np.empty((len(rr), 3), dtype=np.int32)
                    s[:, 0] = det
                    s[:, 1:] = rr
                    segs.append(s)
                    count += len(rr)
            toff.append(count)
        boff.append(len(toff) - 1)
    seg = np.concatenate(segs) if segs else np.zeros((0, 3), dtype=np.int32)
    return seg, np.asarray(toff, dtype=np.int32), np.asarray(boff, dtype=np.int32)


class _DevRanges:
    """so3g_ranges for a thread_intervals argument (None = all samples; a
    DeviceRangesMatrix is used where its segments lie)."""

    def __init__(self, thread_intervals, n_det, n_time):
        self.struct = None
        self.seg_host = None
        self.dev_seg = None
        self.given = thread_intervals is not None
        if isinstance(thread_intervals, DeviceRangesMatrix):
            ti = thread_intervals
            if ti.shape[0] != n_det:
                raise shape_error("thread_intervals", "Expected RangesMatrix with n_det=%d but "
                                  "encountered n_det=%d" % (n_det, ti.shape[0]))
            if ti.shape[1] != n_time:
                raise shape_error("thread_intervals", "Expected RangesMatrix with n_time=%d "
                                  "but encountered n_time=%d" % (n_time, ti.shape[1]))
            self.dev_seg = ti
            return
        bunches = derive_ranges(thread_intervals, n_det, n_time)
        if bunches is None:
            return
        seg, _, _ = flatten_ranges(bunches)
        # Clip to [0, n_time): samples outside the detector's timeline do not
        # exist (the reference would read out of bounds there).
        seg = seg.copy()
        seg[:, 1] = np.clip(seg[:, 1], 0, n_time)
        seg[:, 2] = np.clip(seg[:, 2], 0, n_time)
        self.seg_host = np.ascontiguousarray(seg[seg[:, 2] > seg[:, 1]])

    def upload(self):
        if self.dev_seg is not None:
            d = self.dev_seg
            self.seg = d.seg.to(_device()).contiguous()
            s = _abi.Ranges()
            s.seg = self.seg.data_ptr() if d.n_seg else None
            s.n_seg = d.n_seg
            s.max_len = d.max_len
            self.struct = s
            return self
        seg = self.seg_host
        if seg is None:
            return self
        self.seg = torch.from_numpy(seg).to(_device())
        s = _abi.Ranges()
        s.seg = self.seg.data_ptr() if len(seg) else None
        s.n_seg = len(seg)
        s.max_len = int((seg[:, 2] - seg[:, 1]).max()) if len(seg) else 0
        self.struct = s
        return self

    def ptr(self):
        return self.struct


# ---------------------------------------------------------------------------
# Streaming of host signals.
#
# A signal held in host memory is moved through the device in chunks of
# detector rows, double-buffered: while the kernel of one chunk runs, the
# next chunk is copied in on one copy stream and the previous one copied
# out on another.  The device then holds two chunk buffers instead of the
# whole signal, and the copies overlap the kernels.

STREAM_MIN_BYTES = 64 << 20      # smaller signals go through the device whole
STREAM_CHUNK_BYTES = 128 << 20   # bytes of signal per chunk
_copy_streams = {}


def _streams():
    dev = torch.cuda.current_device()
    if dev not in _copy_streams:
        _copy_streams[dev] = (torch.cuda.Stream(), torch.cuda.Stream())
    return _copy_streams[dev]


def _host_matrix(sig):
    """The host (n_det, n_time) float32 matrix behind a _Signal argument if
    it can be streamed (one contiguous host array, large enough), else
    None."""
    if sig.device_mode or sig.rows is not None or sig._create:
        return None
    a = sig._src
    if isinstance(a, torch.Tensor):
        if a.is_cuda or a.dim() != 2 or not a.is_contiguous():
            return None
        t = a
    else:
        if a.ndim != 2 or not a.flags.c_contiguous or not a.flags.writeable:
            return None
        t = torch.from_numpy(a)
    return t if t.numel() * 4 >= STREAM_MIN_BYTES else None


# A host signal that the device can reach in place -- page-locked memory
# mapped into the device's address space, or ordinary memory on a host whose
# GPUs access pageable memory coherently (a Grace host over NVLink-C2C) --
# can be read and written by the kernels directly: the samples then cross
# the link once, inside the kernel, with no staging buffers.  Measured on a
# GB300 (1000 det x 1M samples, CAR TQU): the copy engines move page-locked
# memory faster than the kernels read it in place (to_map 20.9 ms streamed,
# 25.5 ms in place; from_map 30.1 against 40.7 ms), while a pageable signal
# is read faster in place (to_map 25.8 against 29.3-31.6 ms) but not
# written (from_map 57 against 53-55 ms).  SO3G_GB300_HOST_SIGNAL selects:
#   "auto"   (default) in place where that measured faster: a pageable
#            signal that is only read (to_map);
#   "direct" in place whenever the device can reach the memory;
#   "mapped" in place for page-locked memory only;
#   "stream" never in place.
_HOST_POLICIES = ("auto", "direct", "mapped", "stream")


def host_signal_policy():
    """The host-signal policy named by SO3G_GB300_HOST_SIGNAL."""
    name = os.environ.get("SO3G_GB300_HOST_SIGNAL", "auto")
    if name not in _HOST_POLICIES:
        raise ValueError("SO3G_GB300_HOST_SIGNAL must be one of %s (got %r)"
                         % (", ".join(_HOST_POLICIES), name))
    return name


def _host_mode(host):
    """so3g_host_access mode of the memory of the CPU tensor `host`."""
    _device()
    mode = ctypes.c_int32(0)
    _abi.check(_abi.lib().so3g_host_access(host.data_ptr(), ctypes.byref(mode)),
               "host_access")
    return mode.value


def _host_direct(host, writes):
    """True if the kernels should use the CPU tensor `host` in place under
    host_signal_policy(); `writes`: the call writes the signal."""
    policy = host_signal_policy()
    if policy == "stream":
        return False
    mode = _host_mode(host)
    if policy == "direct":
        return mode != _abi.HOST_NONE
    if policy == "mapped":
        return mode == _abi.HOST_MAPPED
    return mode == _abi.HOST_PAGEABLE and not writes


def _run_host(host, launch, upload, download):
    """launch() over the host signal matrix `host`: in place when
    _host_direct() says so, else streamed through device buffers
    (_stream_rows).  upload=False: the kernels start from zeros instead of
    the contents of `host`.  Returns when the results are in host memory."""
    if host.shape[0] == 0 or host.shape[1] == 0:
        return
    if _host_direct(host, download):
        if not upload:
            host.zero_()
        launch(0, host.shape[0], host)
        torch.cuda.current_stream().synchronize()
        return
    _stream_rows(host, launch, upload, download)


def _stream_rows(host, launch, upload, download):
    """Runs launch(d0, d1, buf) over chunks [d0, d1) of the rows of `host`
    (a CPU float32 (n_det, n_time) tensor), buf being a device copy of
    host[d0:d1] (upload) or zeros, and copies buf back into host[d0:d1]
    afterwards (download).  Returns when every copy is complete."""
    n_det, n_time = host.shape
    if n_det == 0 or n_time == 0:
        return
    dev = _device()
    comp = torch.cuda.current_stream()
    h2d, d2h = _streams()
    pinned = host.is_pinned()
    rows = max(1, min(n_det, STREAM_CHUNK_BYTES // max(1, 4 * n_time)))
    bufs = [torch.empty((rows, n_time), dtype=torch.float32, device=dev) for _ in range(2)]
    h2d.wait_stream(comp)
    freed = [None, None]    # event: the buffer's last use (kernel, download) done
    pending = None          # the chunk to copy out once the next one is launched

    def copy_out(job):
        k, d0, d1, buf, done = job
        with torch.cuda.stream(d2h):
            d2h.wait_event(done)
            host[d0:d1].copy_(buf, non_blocking=pinned)
            out = torch.cuda.Event()
            out.record(d2h)
        freed[k] = out

    for i, d0 in enumerate(range(0, n_det, rows)):
        d1 = min(n_det, d0 + rows)
        k = i % 2
        buf = bufs[k][:d1 - d0]
        with torch.cuda.stream(h2d):
            if freed[k] is not None:
                h2d.wait_event(freed[k])
            if upload:
                buf.copy_(host[d0:d1], non_blocking=pinned)
            else:
                buf.zero_()
            ready = torch.cuda.Event()
            ready.record(h2d)
        comp.wait_event(ready)
        launch(d0, d1, buf)
        done = torch.cuda.Event()
        done.record(comp)
        freed[k] = done
        if pending is not None:
            copy_out(pending)
            pending = None
        if download:
            pending = (k, d0, d1, buf, done)
    if pending is not None:
        copy_out(pending)
    for b in bufs:
        b.record_stream(h2d)
        b.record_stream(d2h)
    comp.wait_stream(h2d)
    comp.wait_stream(d2h)
    comp.synchronize()


# ---------------------------------------------------------------------------
# Maps.

class _MapArg:
    """A map argument: untiled array, or a list of tiles (None = absent),
    resolved to one device buffer plus a tile offset table.  The
    constructor validates; upload() moves the data."""

    def __init__(self, eng, obj, lead, name="map", writable=True):
        self.eng = eng
        self.obj = obj
        self.writable = writable
        self.host = None
        self._host_tiles = None
        self.dev = None
        # The reference checks the component axes of a flat map but not its
        # pixel axes (src/Projection.cxx:867-879, 1055-1082: (ncomp, *, *));
        # a map of another pixel shape is then written out of bounds there.
        # The reference's check runs first, with its message, then the
        # pixel axes are checked too.
        ref_pix = (-1, -1) if not eng._hp else None
        if not eng._tiled:
            arr = as_array(obj, name, "float64")
            if ref_pix:
                _match_shape(name, tuple(lead) + ref_pix, tuple(arr.shape))
            _match_shape(name, tuple(lead) + eng._pix_shape(), tuple(arr.shape))
            self._arr = arr
            return
        if not isinstance(obj, (list, tuple)):
            raise TypeError("Tiled map must be a list of tiles (None for absent tiles)")
        n_tile = eng._n_tile()
        if len(obj) != n_tile:
            raise shape_error(name, "Expected a list of %d tiles but got %d" % (n_tile, len(obj)))
        present = []
        for i, t in enumerate(obj):
            if t is None:
                if eng._populate is not None and eng._populate[i]:
                    raise tiling_error(i, "Projector expects tile but it is missing.")
                continue
            arr = as_array(t, name, "float64")
            if ref_pix:
                _match_shape(name, tuple(lead) + ref_pix, tuple(arr.shape))
            _match_shape(name, tuple(lead) + eng._tile_pix_shape(i), tuple(arr.shape))
            present.append((i, arr))
        self._present = present
        self._n_tile = n_tile

    def upload(self):
        dev = _device()
        self.struct = _abi.Map()
        if not self.eng._tiled:
            arr = self._arr
            if _is_cuda(arr) and arr.is_contiguous():
                self.dev = arr
            else:
                self.dev = to_device(arr, "float64")
                self.host = arr
            self.struct.data = self.dev.data_ptr()
            self.struct.tile_offset = None
            self.struct.n_tile = 0
            return self
        n_tile, present = self._n_tile, self._present
        offsets = np.full(n_tile, -1, dtype=np.int64)
        if present and all(_is_cuda(a) and a.is_contiguous() for _, a in present):
            # Zero-copy: offsets relative to the lowest tile address.
            base = min(a.data_ptr() for _, a in present)
            for i, a in present:
                offsets[i] = (a.data_ptr() - base) // 8
            self.struct.data = base
        else:
            sizes = [a.numel() if isinstance(a, torch.Tensor) else a.size for _, a in present]
            self.dev = torch.empty(max(int(sum(sizes)), 1), dtype=torch.float64, device=dev)
            off = 0
            for (i, a), n in zip(present, sizes):
                offsets[i] = off
                src = a if isinstance(a, torch.Tensor) else torch.from_numpy(
                    np.ascontiguousarray(a))
                self.dev[off:off + n].copy_(src.reshape(-1))
                off += n
            self._host_tiles = present
            self._sizes = sizes
            self.struct.data = self.dev.data_ptr()
        self._tile_table = torch.from_numpy(offsets).to(dev)
        self.struct.tile_offset = self._tile_table.data_ptr()
        self.struct.n_tile = n_tile
        return self

    def writeback(self):
        if not self.writable:
            return
        if self.host is not None:
            copy_back(self.host, self.dev)
        elif self._host_tiles is not None:
            off = 0
            for (i, a), n in zip(self._host_tiles, self._sizes):
                copy_back(a, self.dev[off:off + n])
                off += n


# ---------------------------------------------------------------------------
# Engine classes.

def _as_int(x, what):
    try:
        return int(x.item()) if hasattr(x, "item") else int(x)
    except Exception:
        raise TypeError("Failed to interpret argument \"%s\" as int." % what) from None


# Detector tensors already found free of NaN: the check reads its result
# on the host (a stream synchronisation), which iterative callers passing
# the same tensor call after call need not repeat.  An entry holds while it
# is the same tensor object, storage and version counter (any in-place
# write bumps the version).
_CHECKED = {}
_CHECKED_MAX = 64


def _nan_key(t):
    return (t.data_ptr(), t._version, tuple(t.shape), tuple(t.stride()), str(t.device))


def _nan_checked(t):
    e = _CHECKED.get(id(t))
    return e is not None and e[0]() is t and e[1] == _nan_key(t)


def _remember_checked(t):
    if len(_CHECKED) >= _CHECKED_MAX:
        _CHECKED.clear()
    _CHECKED[id(t)] = (weakref.ref(t), _nan_key(t))


class ProjEngBase:
    """Common machinery of the ProjEng_* classes.  Subclasses fix the
    coordinate system, the pixelization, the tiling, the interpolation and
    the number of spin components."""

    _coord = "CAR"
    _hp = False
    _tiled = False
    _bilinear = False
    _ncomp = 3

    def __init__(self, args):
        args = tuple(args)
        self._populate = None
        if self._hp:
            # Pixelizor_Healpix(bp::object), src/Projection.cxx:534-542, 640-675
            self.nside = _as_int(args[0], "nside")
            nest = bool(args[1])
            self._check_nside(self.nside)
            self.npix = 12 * self.nside * self.nside
            self.nest = nest
            if self._tiled:
                if not nest:
                    raise ValueError("RING not supported for tiled maps")
                self.nside_tile = _as_int(args[2], "nside_tile")
                self._check_nside(self.nside_tile)
                if self.nside_tile > self.nside:
                    raise ValueError("Invalid nside_tile %d > nside %d" % (self.nside_tile,
                                                                          self.nside))
                self.ntiles = 12 * self.nside_tile ** 2
                self.npix_per_tile = self.npix // self.ntiles
                if len(args) >= 4 and args[3] is not None:
                    self._populate = self._populate_from(args[3], self.ntiles)
            return
        # Pixelizor2_Flat(bp::object), src/Projection.cxx:821-829, 971-994
        self.naxis = (_as_int(args[0], "ny"), _as_int(args[1], "nx"))
        self.cdelt = (float(args[2]), float(args[3]))
        self.crpix = (float(args[4]), float(args[5]))
        if self._tiled:
            self.tile_shape = (_as_int(args[6], "tile_y"), _as_int(args[7], "tile_x"))
            if self.tile_shape[0] <= 0 or self.tile_shape[1] <= 0:
                raise ValueError("tile_shape must be positive")
            self.tile_grid = (-(-self.naxis[0] // self.tile_shape[0]),
                              -(-self.naxis[1] // self.tile_shape[1]))
            if len(args) >= 9:
                self._populate = self._populate_from(args[8], self.tile_grid[0] * self.tile_grid[1])

    @staticmethod
    def _populate_from(active, n):
        pop = np.zeros(n, dtype=bool)
        for x in active:
            i = _as_int(x, "active_tiles")
            if 0 <= i < n:
                pop[i] = True
        return pop

    @staticmethod
    def _check_nside(nside):
        if not (0 < nside < 8192 and (nside & (nside - 1)) == 0):
            raise ValueError("Invalid nside %d" % nside)

    # -- reference properties -----------------------------------------------
    @property
    def index_count(self):
        if self._hp:
            return 2 if self._tiled else 1
        return 3 if self._tiled else 2

    @property
    def comp_count(self):
        return self._ncomp

    # -- geometry ---------------------------------------------------------------
    def _pix_shape(self):
        if self._hp:
            return (self.npix,)
        return tuple(self.naxis)

    def _n_tile(self):
        if not self._tiled:
            return 0
        if self._hp:
            return self.ntiles
        return self.tile_grid[0] * self.tile_grid[1]

    def _tile_pix_shape(self, i):
        if self._hp:
            return (self.npix_per_tile,)
        ty, tx = divmod(i, self.tile_grid[1])
        return (min(self.tile_shape[0], self.naxis[0] - ty * self.tile_shape[0]),
                min(self.tile_shape[1], self.naxis[1] - tx * self.tile_shape[1]))

    def _pz(self):
        p = _abi.Pixelization()
        p.coord_sys = _abi.COORD[self._coord]
        p.pix_sys = _abi.PIX_HEALPIX if self._hp else _abi.PIX_FLAT
        p.tiled = 1 if self._tiled else 0
        p.interp = _abi.INTERP_BILINEAR if self._bilinear else _abi.INTERP_NEAREST
        p.n_comp = self._ncomp
        p.pointing = getattr(self, "pointing", DEFAULT_POINTING)
        if self._hp:
            p.nside = self.nside
            p.nest = 1 if self.nest else 0
            if self._tiled:
                p.nside_tile = self.nside_tile
        else:
            p.naxis[0], p.naxis[1] = self.naxis
            p.cdelt[0], p.cdelt[1] = self.cdelt
            p.crpix[0], p.crpix[1] = self.crpix
            if self._tiled:
                p.tile_shape[0], p.tile_shape[1] = self.tile_shape
        return p

    # -- inputs -------------------------------------------------------------------
    def _pointer(self, pbore, pofs):
        """Validates boresight and detector offsets (Pointer<C>::TestInputs,
        src/Projection.cxx:199-226); no device work."""
        bore = as_array(pbore, "boresight", "float64", (-1, 4))
        dets = as_array(pofs, "detectors", "float64", (-1, 4))
        if isinstance(dets, torch.Tensor):
            if not _nan_checked(dets):
                bad = torch.nonzero(torch.isnan(dets).any(dim=1)).flatten().cpu().numpy()
                if not len(bad):
                    _remember_checked(dets)
            else:
                bad = ()
        else:
            bad = np.nonzero(np.isnan(dets).any(axis=1))[0]
        if len(bad):
            raise ValueError("Pointing offset error: nan found at index %d." % bad[0])
        return bore, dets, bore.shape[0], dets.shape[0], _is_cuda(bore)

    @staticmethod
    def _up(*arrs):
        """so3g_init() on this device, then the arrays as device tensors."""
        _ensure_init()
        out = []
        for a, tname in arrs:
            out.append(None if a is None else to_device(a, tname))
        return out

    # -- zeros --------------------------------------------------------------------
    def zeros(self, shape, device=None):
        """Blank map of shape (shape,) + pixel shape; for tiled maps a list
        of tiles (None where the tile is not populated)."""
        if isinstance(shape, (int, np.integer)):
            lead = (int(shape),)
        elif isinstance(shape, tuple):
            lead = tuple(_as_int(s, "shape") for s in shape)
        else:
            return None

        def mk(s):
            if device is not None:
                return torch.zeros(s, dtype=torch.float64, device=device)
            return np.zeros(s, dtype=np.float64)

        if not self._tiled:
            return mk(lead + self._pix_shape())
        if self._populate is None:
            if self._hp:
                raise RuntimeError("Cannot create blank tiled map unless user has specified "
                                   "what tiles to populate.")
            raise shape_error("zeros", "Cannot create blank tiled map unless user has "
                              "specified what tiles to populate.")
        return [mk(lead + self._tile_pix_shape(i)) if self._populate[i] else None
                for i in range(self._n_tile())]

    # -- pointing-only queries ----------------------------------------------------
    def coords(self, pbore, pofs, coord=None):
        """ProjectionEngine::coords (src/Projection.cxx:1316-1349)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        out = _Signal(coord, "coord", "float64", (n_det, n_time, 4), True, dm)
        bore, dets = self._up((bore, "float64"), (dets, "float64"))
        out.upload()
        _abi.check(_abi.lib().so3g_proj_coords(self._pz(), bore.data_ptr(), n_time,
                                               dets.data_ptr(), n_det, out.dev.data_ptr(),
                                               _stream()), "coords")
        out.writeback()
        return out.ret

    def pixels(self, pbore, pofs, pixel=None):
        """ProjectionEngine::pixels (src/Projection.cxx:1351-1385)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        out = _Signal(pixel, "pixel", "int32", (n_det, n_time, self.index_count), True, dm)
        bore, dets = self._up((bore, "float64"), (dets, "float64"))
        out.upload()
        _abi.check(_abi.lib().so3g_proj_pixels(self._pz(), bore.data_ptr(), n_time,
                                               dets.data_ptr(), n_det, out.dev.data_ptr(),
                                               _stream()), "pixels")
        out.writeback()
        return out.ret

    def pointing_matrix(self, pbore, pofs, response, pixel=None, proj=None):
        """ProjectionEngine::pointing_matrix (src/Projection.cxx:1391-1438)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        pix = _Signal(pixel, "pixel", "int32", (n_det, n_time, self.index_count), True, dm)
        pr = _Signal(proj, "proj", "float32", (n_det, n_time, self._ncomp), True, dm)
        resp = as_array(response, "response", "float32", (n_det, 2))
        bore, dets, resp = self._up((bore, "float64"), (dets, "float64"), (resp, "float32"))
        pix.upload()
        pr.upload()
        _abi.check(_abi.lib().so3g_proj_pointing_matrix(
            self._pz(), bore.data_ptr(), n_time, dets.data_ptr(), n_det, resp.data_ptr(),
            pix.dev.data_ptr(), pr.dev.data_ptr(), _stream()), "pointing_matrix")
        pix.writeback()
        pr.writeback()
        return (pix.ret, pr.ret)

    def tile_hits(self, pbore, pofs):
        """ProjectionEngine::tile_hits (src/Projection.cxx:1543-1601)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        if not self._tiled:
            raise RuntimeError("No tiles in this pixelization.")
        n_tile = self._n_tile()
        bore, dets = self._up((bore, "float64"), (dets, "float64"))
        hits = torch.zeros(n_tile, dtype=torch.int64, device=_device())
        _abi.check(_abi.lib().so3g_proj_tile_hits(self._pz(), bore.data_ptr(), n_time,
                                                  dets.data_ptr(), n_det, hits.data_ptr(),
                                                  n_tile, _stream()), "tile_hits")
        return [int(x) for x in hits.cpu().numpy()]

    def _domain_ranges(self, bore, dets, n_time, n_det, mode, n_domain, dmap=None,
                       tile_domain=None):
        bore, dets = self._up((bore, "float64"), (dets, "float64"))
        lib = _abi.lib()
        err = _ErrRecord()
        n_edges = torch.zeros(1, dtype=torch.int64, device=_device())
        cap = max(1024, 4 * n_det)
        td = None
        n_tile = self._n_tile()
        if tile_domain is not None:
            td = torch.from_numpy(np.asarray(tile_domain, dtype=np.int32)).to(_device())
        mstruct = None
        if dmap is not None:
            mstruct = dmap.upload().struct
        while True:
            edges = torch.empty((cap, 3), dtype=torch.int32, device=_device())
            n_edges.zero_()
            _abi.check(lib.so3g_proj_domain_edges(
                self._pz(), bore.data_ptr(), n_time, dets.data_ptr(), n_det, mode, n_domain,
                mstruct, _ptr(td), n_tile, edges.data_ptr(), cap, n_edges.data_ptr(),
                err.ptr, _stream()), "domain ranges")
            n = int(n_edges.item())
            if n <= cap:
                break
            cap = n
        err.raise_if_set()
        e = edges[:n].cpu().numpy()
        return _edges_to_ranges(e, n_det, n_time, n_domain)

    def pixel_ranges(self, pbore, pofs, map=None, n_domain=-1):
        """ProjectionEngine::pixel_ranges (src/Projection.cxx:1440-1541):
        [[Ranges per det] per domain] for the parallel bunch and one serial
        pseudo-domain for samples whose taps span domains."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        dmap = None
        if map is not None:
            dmap = _MapArg(self, map, (self._ncomp,), writable=False)
        n_domain = int(n_domain)
        if n_domain <= 0:
            from . import useful_info
            n_domain = useful_info()["omp_num_threads"]
        return self._domain_ranges(bore, dets, n_time, n_det, 1 if dmap is not None else 0,
                                   n_domain, dmap=dmap)

    def tile_ranges(self, pbore, pofs, tile_lists):
        """ProjectionEngine::tile_ranges (src/Projection.cxx:1606-1705)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        if not self._tiled:
            raise RuntimeError("No tiles in this pixelization.")
        n_tile = self._n_tile()
        thread_idx = np.full(n_tile, -1, dtype=np.int32)
        for i, tl in enumerate(tile_lists):
            for t in tl:
                thread_idx[_as_int(t, "tile")] = i
        return self._domain_ranges(bore, dets, n_time, n_det, 2, len(tile_lists),
                                   tile_domain=thread_idx)

    # -- projection operators -----------------------------------------------------
    def from_map(self, map, pbore, pofs, response, signal=None):
        """ProjectionEngine::from_map (src/Projection.cxx:1728-1770)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        m = _MapArg(self, map, (self._ncomp,), writable=False)
        sig = _Signal(signal, "signal", "float32", (n_det, n_time), True, dm)
        resp = as_array(response, "response", "float32", (n_det, 2))
        bore, dets, resp = self._up((bore, "float64"), (dets, "float64"), (resp, "float32"))
        m.upload()
        err = _ErrRecord()
        lib, pz = _abi.lib(), self._pz()

        def launch(d0, d1, buf):
            _abi.check(lib.so3g_proj_from_map(
                pz, bore.data_ptr(), n_time, dets.data_ptr() + 32 * d0, d1 - d0,
                resp.data_ptr() + 8 * d0, m.struct, buf.data_ptr(), buf.stride(0), err.ptr,
                _stream()), "from_map")

        host = _host_matrix(sig)
        if host is not None:
            _run_host(host, launch, upload=True, download=True)
            err.raise_if_set()
            return sig.ret
        if sig._create and not sig.device_mode and 4 * n_det * n_time >= STREAM_MIN_BYTES:
            # A new host signal (signal=None): page-locked (torch caches
            # such blocks across calls), filled by zeroed device chunks and
            # copied out; nothing is copied in.
            out = torch.empty((n_det, n_time), dtype=torch.float32, pin_memory=True)
            _run_host(out, launch, upload=False, download=True)
            err.raise_if_set()
            return list(out.numpy())
        sig.upload()
        launch(0, n_det, sig.dev)
        err.raise_if_set()
        sig.writeback()
        return sig.ret

    def to_map(self, map, pbore, pofs, response, signal, det_weights=None,
               thread_intervals=None, accum=None):
        """ProjectionEngine::to_map (src/Projection.cxx:1924-1966)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        if map is None:
            map = self.zeros(self._ncomp, device=_device() if dm else None)
        m = _MapArg(self, map, (self._ncomp,))
        sig = _Signal(signal, "signal", "float32", (n_det, n_time), False, dm)
        w = as_array(det_weights, "det_weights", "float32", (n_det,), optional=True)
        resp = as_array(response, "response", "float32", (n_det, 2))
        rng = _DevRanges(thread_intervals, n_det, n_time)
        bore, dets, resp, w = self._up((bore, "float64"), (dets, "float64"),
                                       (resp, "float32"), (w, "float32"))
        m.upload()
        err = _ErrRecord()
        lib, pz = _abi.lib(), self._pz()
        acc = DEFAULT_ACCUM if accum is None else accum
        host = _host_matrix(sig) if not rng.given else None
        if host is not None:
            def launch(d0, d1, buf):
                _abi.check(lib.so3g_proj_to_map(
                    pz, bore.data_ptr(), n_time, dets.data_ptr() + 32 * d0, d1 - d0,
                    resp.data_ptr() + 8 * d0, buf.data_ptr(), buf.stride(0),
                    None if w is None else w.data_ptr() + 4 * d0, None, m.struct, acc,
                    err.ptr, _stream()), "to_map")

            _run_host(host, launch, upload=True, download=False)
        else:
            sig.upload()
            rng.upload()
            _abi.check(lib.so3g_proj_to_map(
                pz, bore.data_ptr(), n_time, dets.data_ptr(), n_det, resp.data_ptr(),
                sig.dev.data_ptr(), sig.det_stride, _ptr(w), rng.ptr(), m.struct, acc,
                err.ptr, _stream()), "to_map")
        err.raise_if_set()
        m.writeback()
        return map

    def to_weight_map(self, map, pbore, pofs, response, det_weights=None,
                      thread_intervals=None, accum=None):
        """ProjectionEngine::to_weight_map (src/Projection.cxx:1968-2010)."""
        bore, dets, n_time, n_det, dm = self._pointer(pbore, pofs)
        if map is None:
            map = self.zeros((self._ncomp, self._ncomp), device=_device() if dm else None)
        m = _MapArg(self, map, (self._ncomp, self._ncomp))
        w = as_array(det_weights, "det_weights", "float32", (n_det,), optional=True)
        resp = as_array(response, "response", "float32", (n_det, 2))
        rng = _DevRanges(thread_intervals, n_det, n_time)
        bore, dets, resp, w = self._up((bore, "float64"), (dets, "float64"),
                                       (resp, "float32"), (w, "float32"))
        m.upload()
        rng.upload()
        err = _ErrRecord()
        _abi.check(_abi.lib().so3g_proj_to_weight_map(
            self._pz(), bore.data_ptr(), n_time, dets.data_ptr(), n_det, resp.data_ptr(),
            _ptr(w), rng.ptr(), m.struct, DEFAULT_ACCUM if accum is None else accum,
            err.ptr, _stream()), "to_weight_map")
        err.raise_if_set()
        m.writeback()
        return map


def _edges_to_ranges(e, n_det, n_time, n_domain):
    """Domain edge records (det, t, label) -> [parallel, serial] nested
    lists of RangesInt32, built as pixel_ranges/tile_ranges do
    (src/Projection.cxx:1507-1523)."""
    par = [[RangesInt32(n_time) for _ in range(n_det)] for _ in range(n_domain)]
    ser = [[RangesInt32(n_time) for _ in range(n_det)]]
    if len(e):
        order = np.lexsort((e[:, 1], e[:, 0]))
        e = e[order]
        ends = np.full(len(e), n_time, dtype=np.int64)
        same = e[1:, 0] == e[:-1, 0]
        ends[:-1][same] = e[1:, 1][same]
        keep = e[:, 2] >= 0
        det, t, lab, ends = e[keep, 0], e[keep, 1], e[keep, 2], ends[keep]
        # Domain index n_domain: the serial (shared) ranges.
        tgt = np.minimum(lab, n_domain).astype(np.int64)
        # Group by (domain, detector); within a group the intervals stay in
        # time order (the stable sort keeps the (det, t) order).
        key = tgt * n_det + det
        g = np.argsort(key, kind="stable")
        key, pairs = key[g], np.stack([t[g].astype(np.int64), ends[g]], axis=1)
        cut = np.flatnonzero(np.diff(key)) + 1
        starts = np.concatenate([[0], cut])
        stops = np.concatenate([cut, [len(key)]])
        # Millions of small interval lists: the cyclic garbage collector
        # would rescan the growing heap many times over while they are made.
        was_enabled = gc.isenabled()
        gc.disable()
        try:
            for a, b in zip(starts.tolist(), stops.tolist()):
                d, k = divmod(int(key[a]), n_det)
                target = par[d] if d < n_domain else ser[0]
                target[k]._set(pairs[a:b])
        finally:
            if was_enabled:
                gc.enable()
    return [par, ser]


# ---------------------------------------------------------------------------
# ProjEng_Precomp (src/Projection.cxx:2012-2256).

class ProjEngPrecompBase:
    """Projection with precomputed pixel indices and spin factors."""

    _tiled = False

    def __init__(self, *args):
        pass

    def _inputs(self, pixel_index, spin_proj, device_mode):
        n_idx = 3 if self._tiled else 2
        pix = _Signal(pixel_index, "pixel_index", "int32", (-1, -1, -1), False, device_mode)
        n_det, n_time, n_pix = pix.dims
        if n_pix != n_idx:
            raise shape_error("pixel_index", "Expected %d pixel indices per sample but got %d"
                              % (n_idx, n_pix))
        sp = _Signal(spin_proj, "spin_proj", "float32", (n_det, n_time, -1), False, device_mode)
        n_spin = sp.dims[2]
        if not 1 <= n_spin <= 3:
            raise shape_error("spin_proj", "Expected 1, 2 or 3 spin components but got %d"
                              % n_spin)
        return pix, sp, n_det, n_time, n_spin

    @staticmethod
    def _upload(pix, sp):
        _ensure_init()
        pix.upload()
        sp.upload()
        pix.dev = pix.dev.contiguous()
        sp.dev = sp.dev.contiguous()

    def _map(self, obj, lead, writable=True):
        g = _abi.PrecompGeom()
        g.tiled = 1 if self._tiled else 0
        g.n_comp = lead[0]
        if not self._tiled:
            arr = as_array(obj, "map", "float64", tuple(lead) + (-1, -1))
            g.naxis[0], g.naxis[1] = arr.shape[-2], arr.shape[-1]
            return g, _PcMap(arr, writable)
        if not isinstance(obj, (list, tuple)):
            raise TypeError("Tiled map must be a list of tiles (None for absent tiles)")
        dims = np.zeros((len(obj), 2), dtype=np.int32)
        for i, t in enumerate(obj):
            if t is not None:
                a = as_array(t, "map", "float64", tuple(lead) + (-1, -1))
                dims[i] = a.shape[-2:]
        holder = _PcMap(list(obj), writable, tiled=True)
        holder.tile_dims_host = dims
        return g, holder

    def from_map(self, map, pixel_index, spin_proj, signal=None):
        """ProjEng_Precomp::from_map (src/Projection.cxx:2036-2085)."""
        dm = _is_cuda(pixel_index)
        pix, sp, n_det, n_time, n_spin = self._inputs(pixel_index, spin_proj, dm)
        g, m = self._map(map, (n_spin,), writable=False)
        sig = _Signal(signal, "signal", "float32", (n_det, n_time), True, dm)
        self._upload(pix, sp)
        m.upload(g)
        sig.upload()
        err = _ErrRecord()
        _abi.check(_abi.lib().so3g_precomp_from_map(
            g, pix.dev.data_ptr(), sp.dev.data_ptr(), n_det, n_time, m.struct,
            sig.dev.data_ptr(), sig.det_stride, err.ptr, _stream()), "precomp from_map")
        err.raise_if_set()
        sig.writeback()
        return sig.ret

    def to_map(self, map, pixel_index, spin_proj, signal, det_weights=None,
               thread_intervals=None, accum=None):
        """ProjEng_Precomp::to_map (src/Projection.cxx:2157-2206)."""
        dm = _is_cuda(pixel_index)
        pix, sp, n_det, n_time, n_spin = self._inputs(pixel_index, spin_proj, dm)
        g, m = self._map(map, (n_spin,))
        sig = _Signal(signal, "signal", "float32", (n_det, n_time), False, dm)
        w = as_array(det_weights, "det_weights", "float32", (n_det,), optional=True)
        rng = _DevRanges(thread_intervals, n_det, n_time)
        self._upload(pix, sp)
        m.upload(g)
        sig.upload()
        rng.upload()
        w = None if w is None else to_device(w, "float32")
        err = _ErrRecord()
        _abi.check(_abi.lib().so3g_precomp_to_map(
            g, pix.dev.data_ptr(), sp.dev.data_ptr(), n_det, n_time, sig.dev.data_ptr(),
            sig.det_stride, _ptr(w), rng.ptr(), m.struct,
            DEFAULT_ACCUM if accum is None else accum, err.ptr, _stream()), "precomp to_map")
        err.raise_if_set()
        m.writeback()
        return map

    def to_weight_map(self, map, pixel_index, spin_proj, det_weights=None,
                      thread_intervals=None, accum=None):
        """ProjEng_Precomp::to_weight_map (src/Projection.cxx:2208-2253)."""
        dm = _is_cuda(pixel_index)
        pix, sp, n_det, n_time, n_spin = self._inputs(pixel_index, spin_proj, dm)
        g, m = self._map(map, (n_spin, n_spin))
        w = as_array(det_weights, "det_weights", "float32", (n_det,), optional=True)
        rng = _DevRanges(thread_intervals, n_det, n_time)
        self._upload(pix, sp)
        m.upload(g)
        rng.upload()
        w = None if w is None else to_device(w, "float32")
        err = _ErrRecord()
        _abi.check(_abi.lib().so3g_precomp_to_weight_map(
            g, pix.dev.data_ptr(), sp.dev.data_ptr(), n_det, n_time, _ptr(w), rng.ptr(),
            m.struct, DEFAULT_ACCUM if accum is None else accum, err.ptr, _stream()),
            "precomp to_weight_map")
        err.raise_if_set()
        m.writeback()
        return map


class _PcMap:
    """Map holder for the precomputed-pointing engines (validated by the
    caller; upload() moves the data)."""

    def __init__(self, obj, writable, tiled=False):
        self.obj = obj
        self.writable = writable
        self.tiled = tiled
        self.host = None
        self._tiles = None
        self.tile_dims_host = None

    def upload(self, g):
        dev = _device()
        self.struct = _abi.Map()
        obj = self.obj
        if not self.tiled:
            if _is_cuda(obj) and obj.is_contiguous():
                self.dev = obj
            else:
                self.dev = to_device(obj, "float64")
                self.host = obj
            self.struct.data = self.dev.data_ptr()
            return self
        offsets = np.full(len(obj), -1, dtype=np.int64)
        present = [(i, t) for i, t in enumerate(obj) if t is not None]
        sizes = [(t.numel() if isinstance(t, torch.Tensor) else np.asarray(t).size)
                 for _, t in present]
        self.dev = torch.empty(max(1, int(sum(sizes))), dtype=torch.float64, device=dev)
        off = 0
        for (i, t), n in zip(present, sizes):
            offsets[i] = off
            src = t if isinstance(t, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(t))
            self.dev[off:off + n].copy_(src.reshape(-1))
            off += n
        self._tiles = present
        self._sizes = sizes
        self._offsets = torch.from_numpy(offsets).to(dev)
        self._dims = torch.from_numpy(self.tile_dims_host).to(dev)
        g.tile_dims = self._dims.data_ptr()
        self.struct.data = self.dev.data_ptr()
        self.struct.tile_offset = self._offsets.data_ptr()
        self.struct.n_tile = len(obj)
        return self

    def writeback(self):
        if not self.writable:
            return
        if self.host is not None:
            copy_back(self.host, self.dev)
        elif self._tiles is not None:
            off = 0
            for (i, t), n in zip(self._tiles, self._sizes):
                copy_back(t, self.dev[off:off + n])
                off += n


# ---------------------------------------------------------------------------
# The class family (src/Projection.cxx:2258-2358).

SPINS = {"T": 1, "QU": 2, "TQU": 3}
COORDS = ["Flat", "Quat", "CAR", "CEA", "ARC", "SIN", "TAN", "ZEA"]


def _make_classes():
    out = {}
    for coord in COORDS:
        for spin, nc in SPINS.items():
            for tiling in ("Tiled", "NonTiled"):
                for bil in (False, True):
                    name = "ProjEng_%s_%s_%s%s" % (coord, spin, tiling, "_Bilinear" if bil else "")
                    out[name] = type(name, (ProjEngBase,), dict(
                        _coord=coord, _hp=False, _tiled=(tiling == "Tiled"), _bilinear=bil,
                        _ncomp=nc, __doc__="%s engine (GB300)." % name))
    for spin, nc in SPINS.items():
        for tiling in ("NonTiled", "Tiled"):
            name = "ProjEng_HP_%s_%s" % (spin, tiling)
            out[name] = type(name, (ProjEngBase,), dict(
                _coord="CAR", _hp=True, _tiled=(tiling == "Tiled"), _bilinear=False,
                _ncomp=nc, __doc__="%s engine (GB300)." % name))
    for tiling in ("NonTiled", "Tiled"):
        name = "ProjEng_Precomp_%s" % tiling
        out[name] = type(name, (ProjEngPrecompBase,), dict(
            _tiled=(tiling == "Tiled"), __doc__="%s engine (GB300)." % name))
    return out


ENGINES = _make_classes()
globals().update(ENGINES)
