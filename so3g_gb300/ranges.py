"""Interval lists: RangesInt32 and RangesMatrix.

RangesInt32 follows the semantics of so3g's Ranges<int32_t>
(include/Ranges.h:14-65, src/Ranges.cxx): a sample count plus a list of
half-open [start, end) intervals.  add_interval() merges; the thread
assignment routines build their lists with append_interval_no_check(),
which does not.  RangesMatrix follows python/proj/ranges.py:11-297: a
nested container of Ranges whose last axis is the sample axis.

These are host-side containers (the argument type of ``thread_intervals``),
kept in numpy arrays; the projection kernels receive them flattened to
(det, start, end) segments.
"""
import numpy as np


_NO_SEGS = np.zeros((0, 2), dtype=np.int64)


class RangesInt32:
    """Half-open intervals over ``count`` samples.

    The intervals live in an (n, 2) int64 numpy array; intervals added one
    at a time (append_interval_no_check, as the thread assignment loops do)
    collect in a short Python list that is folded into the array when the
    intervals are next read, so neither appending nor reading costs a
    Python object per interval."""

    def __init__(self, count=0, reference=0):
        self.count = int(count)
        self.reference = int(reference)
        self._a = _NO_SEGS
        self._tail = []   # [start, end] pairs appended since the last fold

    def _arr(self):
        """The intervals as an (n, 2) int64 array, in storage order."""
        if self._tail:
            t = np.asarray(self._tail, dtype=np.int64).reshape(-1, 2)
            self._a = np.concatenate([self._a, t]) if len(self._a) else t
            self._tail = []
        return self._a

    def _set(self, pairs):
        self._a = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
        self._tail = []

    @property
    def _segs(self):
        """The intervals as a list of [start, end] lists."""
        return self._arr().tolist()

    @_segs.setter
    def _segs(self, pairs):
        self._set(pairs)

    # -- construction --------------------------------------------------------
    @classmethod
    def from_array(cls, intervals, count):
        r = cls(count)
        r._set(intervals)
        r._cleanup()
        return r

    @classmethod
    def from_mask(cls, mask):
        mask = np.asarray(mask, dtype=bool)
        if mask.ndim != 1:
            return RangesMatrix([cls.from_mask(m) for m in mask])
        r = cls(len(mask))
        if len(mask):
            d = np.diff(mask.astype(np.int8), prepend=np.int8(0), append=np.int8(0))
            r._set(np.stack([np.flatnonzero(d == 1), np.flatnonzero(d == -1)], axis=1))
        return r

    def copy(self):
        r = RangesInt32(self.count, self.reference)
        r._a = self._arr().copy()
        return r

    def zeros_like(self):
        return RangesInt32(self.count, self.reference)

    def ones_like(self):
        r = RangesInt32(self.count, self.reference)
        if self.count > 0:
            r._set([[0, self.count]])
        return r

    # -- basic operations ------------------------------------------------------
    def append_interval_no_check(self, start, end):
        self._tail.append([int(start), int(end)])
        return self

    def add_interval(self, start, end):
        self._tail.append([int(start), int(end)])
        self._cleanup()
        return self

    def _cleanup(self):
        """Clips to [0, count), drops empty intervals, sorts and merges the
        overlapping or touching ones."""
        a = self._arr()
        if not len(a):
            return
        lo = np.maximum(a[:, 0], 0)
        hi = np.minimum(a[:, 1], self.count)
        keep = hi > lo
        lo, hi = lo[keep], hi[keep]
        if not len(lo):
            self._a = _NO_SEGS
            return
        o = np.lexsort((hi, lo))
        lo, hi = lo[o], hi[o]
        # An interval opens a new run when it starts past every earlier end.
        new = np.empty(len(lo), dtype=bool)
        new[0] = True
        new[1:] = lo[1:] > np.maximum.accumulate(hi)[:-1]
        first = np.flatnonzero(new)
        self._a = np.stack([lo[first], np.maximum.reduceat(hi, first)], axis=1)

    def merge(self, src):
        a = src._arr()
        if len(a):
            self._tail.extend(a.tolist())
        self._cleanup()
        return self

    def intersect(self, src):
        self._set((self * src)._arr())
        return self

    def complement(self):
        out = RangesInt32(self.count, self.reference)
        a = self._arr()
        if not len(a):
            if self.count > 0:
                out._set([[0, self.count]])
            return out
        o = np.lexsort((a[:, 1], a[:, 0]))
        lo, hi = a[o, 0], a[o, 1]
        # x before interval i: the largest end so far (0 at the start).
        x = np.maximum.accumulate(np.concatenate([[0], hi]))
        gap = lo > x[:-1]
        pairs = np.stack([x[:-1][gap], lo[gap]], axis=1)
        if x[-1] < self.count:
            pairs = np.concatenate([pairs, [[x[-1], self.count]]])
        out._set(pairs)
        return out

    def buffer(self, buff):
        a = self._arr()
        self._set(a + np.array([-int(buff), int(buff)], dtype=np.int64))
        self._cleanup()
        return self

    def buffered(self, buff):
        return self.copy().buffer(buff)

    def close_gaps(self, gap):
        segs = sorted(self._segs)
        out = []
        for a, b in segs:
            if out and a - out[-1][1] <= gap:
                out[-1][1] = max(out[-1][1], b)
            else:
                out.append([a, b])
        self._set(out)
        return self

    # -- views -----------------------------------------------------------------
    def ranges(self):
        """(n, 2) int32 array of [start, end) pairs."""
        return self._arr().astype(np.int32)

    def mask(self):
        m = np.zeros(self.count + 1, dtype=np.int32)
        a = self._arr()
        if len(a):
            lo = np.clip(a[:, 0], 0, self.count)
            hi = np.clip(a[:, 1], 0, self.count)
            keep = hi > lo
            np.add.at(m, lo[keep], 1)
            np.add.at(m, hi[keep], -1)
        return np.cumsum(m[:-1]) > 0

    @property
    def shape(self):
        return (self.count,)

    def __len__(self):
        return self.count

    def __invert__(self):
        return self.complement()

    def __neg__(self):
        return self.complement()

    def __add__(self, other):
        return self.copy().merge(other)

    def __mul__(self, other):
        out = []
        a = sorted(self._segs)
        b = sorted(other._segs)
        i = j = 0
        while i < len(a) and j < len(b):
            lo = max(a[i][0], b[j][0])
            hi = min(a[i][1], b[j][1])
            if hi > lo:
                out.append([lo, hi])
            if a[i][1] < b[j][1]:
                i += 1
            else:
                j += 1
        r = RangesInt32(self.count, self.reference)
        r._set(out)
        return r

    def __getitem__(self, index):
        if not isinstance(index, slice):
            raise IndexError("RangesInt32 supports slice indexing only")
        start, stop, step = index.indices(self.count)
        if step != 1:
            raise IndexError("RangesInt32 slices must have unit step")
        out = RangesInt32(max(0, stop - start), self.reference + start)
        a = self._arr()
        if len(a):
            lo = np.maximum(a[:, 0], start) - start
            hi = np.minimum(a[:, 1], stop) - start
            keep = hi > lo
            out._set(np.stack([lo[keep], hi[keep]], axis=1))
        return out

    def __repr__(self):
        return "RangesInt32(n=%d:rngs=%d)" % (self.count, len(self._arr()))


class RangesMatrix:
    """A grid of RangesInt32 objects (python/proj/ranges.py:11-297)."""

    def __init__(self, items=(), child_shape=None, skip_shape_check=False):
        self.ranges = [x for x in items]
        if len(self.ranges):
            child_shape = self.ranges[0].shape
            if not skip_shape_check:
                assert all(item.shape == child_shape for item in self.ranges)
        elif child_shape is None:
            child_shape = ()
        self._child_shape = tuple(child_shape)

    @property
    def shape(self):
        if not self.ranges:
            return (0,) + self._child_shape
        return (len(self.ranges),) + tuple(self.ranges[0].shape)

    def __len__(self):
        return self.shape[0]

    def __iter__(self):
        return iter(self.ranges)

    def __repr__(self):
        return "RangesMatrix(" + ",".join(map(str, self.shape)) + ")"

    def copy(self):
        return RangesMatrix([x.copy() for x in self.ranges], child_shape=self.shape[1:])

    def zeros_like(self):
        return RangesMatrix([x.zeros_like() for x in self.ranges], child_shape=self.shape[1:])

    def ones_like(self):
        return RangesMatrix([x.ones_like() for x in self.ranges], child_shape=self.shape[1:])

    def mask(self, dest=None):
        if not self.ranges:
            out = np.zeros(self.shape, dtype=bool)
        else:
            out = np.array([r.mask() for r in self.ranges])
        if dest is not None:
            dest[...] = out
            return dest
        return out

    def __getitem__(self, index):
        if isinstance(index, tuple):
            if len(index) == 0:
                return self
            head, rest = index[0], index[1:]
        else:
            head, rest = index, ()
        if isinstance(head, (int, np.integer)):
            item = self.ranges[int(head)]
            return item[rest] if rest else item
        if isinstance(head, slice):
            items = self.ranges[head]
        else:
            sel = np.arange(len(self.ranges))[head]
            items = [self.ranges[i] for i in np.atleast_1d(sel)]
        if rest:
            items = [x[rest if len(rest) > 1 else rest[0]] for x in items]
        return RangesMatrix(items, child_shape=self.shape[1:])

    def __invert__(self):
        return RangesMatrix([~x for x in self.ranges], child_shape=self.shape[1:])

    def __mul__(self, other):
        if isinstance(other, RangesMatrix) and len(other.shape) == len(self.shape):
            return RangesMatrix([a * b for a, b in zip(self.ranges, other.ranges)],
                                child_shape=self.shape[1:])
        return RangesMatrix([a * other for a in self.ranges], child_shape=self.shape[1:])

    def __add__(self, other):
        if isinstance(other, RangesMatrix) and len(other.shape) == len(self.shape):
            return RangesMatrix([a + b for a, b in zip(self.ranges, other.ranges)],
                                child_shape=self.shape[1:])
        return RangesMatrix([a + other for a in self.ranges], child_shape=self.shape[1:])

    @classmethod
    def zeros(cls, shape):
        shape = tuple(shape)
        if len(shape) == 1:
            return RangesInt32(shape[0])
        return cls([cls.zeros(shape[1:]) for _ in range(shape[0])], child_shape=shape[1:])

    @classmethod
    def ones(cls, shape):
        shape = tuple(shape)
        if len(shape) == 1:
            return RangesInt32(shape[0]).ones_like()
        return cls([cls.ones(shape[1:]) for _ in range(shape[0])], child_shape=shape[1:])

    @classmethod
    def from_mask(cls, mask):
        if _is_cuda(mask) and mask.dim() == 2:
            return DeviceRangesMatrix.from_mask(mask)
        mask = np.asarray(mask, dtype=bool)
        if mask.ndim == 1:
            return RangesInt32.from_mask(mask)
        return cls([cls.from_mask(m) for m in mask], child_shape=mask.shape[1:])


def _is_cuda(x):
    import sys
    torch = sys.modules.get("torch")
    return torch is not None and isinstance(x, torch.Tensor) and x.is_cuda


class DeviceRangesMatrix:
    """An (n_det, n_time) RangesMatrix held on the device as (det, start,
    end) segments, built from a CUDA mask by RangesMatrix.from_mask
    (so3g_mask_count_segments / so3g_mask_fill_segments) without a trip to
    the host.  Passed as thread_intervals (one thread, a RangesMatrix
    (ndet) in the reference's terms) its segments go to the projection
    kernels where they lie; to_host() gives the RangesMatrix itself."""

    def __init__(self, seg, n_det, n_time, max_len):
        self.seg = seg              # (n_seg, 3) int32 CUDA tensor
        self.n_seg = int(seg.shape[0])
        self.max_len = int(max_len)
        self._shape = (int(n_det), int(n_time))

    @classmethod
    def from_mask(cls, mask):
        import torch
        from . import _abi
        from .projeng import _stream
        if mask.dim() != 2:
            raise ValueError("expected an (n_det, n_time) mask, got shape %s"
                             % (tuple(mask.shape),))
        dev = mask.device
        with torch.cuda.device(dev):
            m = mask
            if m.dtype != torch.bool and m.dtype != torch.uint8:
                m = m != 0
            if m.stride(1) != 1:
                m = m.contiguous()
            m8 = m.view(torch.uint8) if m.dtype == torch.bool else m
            n_det, n_time = m8.shape
            lib, st = _abi.lib(), _stream()
            counts = torch.zeros(n_det, dtype=torch.int32, device=dev)
            _abi.check(lib.so3g_mask_count_segments(m8.data_ptr(), n_det, n_time, m8.stride(0),
                                                    counts.data_ptr(), st),
                       "mask_count_segments")
            first = torch.cumsum(counts, 0, dtype=torch.int64) - counts
            n_seg = int(counts.sum()) if n_det else 0
            seg = torch.empty((n_seg, 3), dtype=torch.int32, device=dev)
            max_len = torch.zeros(1, dtype=torch.int32, device=dev)
            if n_seg:
                _abi.check(lib.so3g_mask_fill_segments(m8.data_ptr(), n_det, n_time,
                                                       m8.stride(0), first.data_ptr(),
                                                       counts.data_ptr(), seg.data_ptr(),
                                                       max_len.data_ptr(), st),
                           "mask_fill_segments")
            return cls(seg, n_det, n_time, int(max_len.item()))

    @property
    def shape(self):
        return self._shape

    def __len__(self):
        return self._shape[0]

    def __repr__(self):
        return "DeviceRangesMatrix(%d,%d; %d segments)" % (self._shape + (self.n_seg,))

    def to_host(self):
        """The same ranges as a (host) RangesMatrix."""
        seg = self.seg.cpu().numpy()
        n_det, n_time = self._shape
        rows = [RangesInt32(n_time) for _ in range(n_det)]
        for d, a, b in seg:
            rows[int(d)].append_interval_no_check(int(a), int(b))
        return RangesMatrix(rows, child_shape=(n_time,))

    def mask(self, dest=None):
        return self.to_host().mask(dest)

    def __getitem__(self, index):
        return self.to_host()[index]

    def __iter__(self):
        return iter(self.to_host())


def wrap_ivals(ivals):
    """Nested lists of RangesInt32 [bunch][thread][det] -> list of
    RangesMatrix (python/proj/wcs.py:887-915)."""
    return [RangesMatrix([RangesMatrix(y) for y in x]) for x in ivals]
