"""Map-geometry front end of the ProjEng classes: the Projectionist API of
so3g.proj (python/proj/wcs.py), so that map-making code written against
so3g runs on the GB300 engines.

A Projectionist is a pixelization plus the rotation from celestial to the
projection's native frame (``q_celestial_to_native``).  Every map
operation takes an Assembly -- boresight quaternions ``Q`` (focal plane
-> celestial) and a FocalPlane (detector -> focal plane quaternions and
(T, P) responses) -- and becomes one call of a ProjEng method with
``q_native = q_celestial_to_native * Q``, the detector quaternions and the
responses.  q_native is cached per boresight object; a boresight held on
the GPU is rotated there.

Two geometries:
- ``_FlatGeometry`` (Projectionist): a (ny, nx) pixel grid with CDELT (in
  radians) and CRPIX of a FITS-style celestial WCS, optionally cut into
  tiles of ``tile_shape`` pixels;
- ``_HealpixGeometry`` (ProjectionistHealpix): nside, ordering and
  optional tiling by nside_tile.

Thread assignments are accepted in every form so3g accepts.  The GPU
kernels accumulate with atomics, so an assignment only selects samples:
'domdir' gives the 'simple' stripes.
"""
import heapq

import numpy as np

from . import quat
from . import mapthreads
from ..ranges import RangesMatrix, RangesInt32, wrap_ivals  # noqa: F401

Ranges = RangesInt32

#: Interpolation names; the first is the default.
INTERPOLS = ['nearest', 'bilinear']
THREAD_ASSIGNMENT_METHODS = ['simple', 'domdir', 'tiles']
THREAD_ASSIGNMENT_METHODS_HP = ['simple', 'tiles']

_COMPS_BY_COUNT = {1: 'T', 2: 'QU', 3: 'TQU'}
_INTERP_SUFFIX = {'nearest': '', 'nn': '', 'bilinear': '_Bilinear', 'lin': '_Bilinear'}


def _engines():
    import so3g_gb300
    return so3g_gb300


def engine_class_name(proj, comps, tiled, interpol):
    """Name of the ProjEng class for a projection, component set, tiling
    and interpolation ('ProjEng_CAR_TQU_NonTiled_Bilinear', ...)."""
    if interpol not in _INTERP_SUFFIX:
        raise ValueError("ProjEng interpol '%s' not recognized" % str(interpol))
    return 'ProjEng_%s_%s_%s%s' % (proj, comps, 'Tiled' if tiled else 'NonTiled',
                                   _INTERP_SUFFIX[interpol])


def lpt_groups(loads, items, n_groups):
    """Longest-processing-time grouping: items in decreasing load (ties:
    decreasing item), each to the group with the least load so far (ties:
    the lowest group).  Returns the item lists of the n_groups groups."""
    groups = [[] for _ in range(n_groups)]
    heap = [(0, g) for g in range(n_groups)]
    for load, item in sorted(zip(loads, items), reverse=True):
        total, g = heapq.heappop(heap)
        groups[g].append(item)
        heapq.heappush(heap, (total + load, g))
    return groups


def _first_tile_shape(m):
    """Shape of a map: an array, or the first present tile of a tile list."""
    if not isinstance(m, list):
        return tuple(m.shape)
    shapes = [tuple(t.shape) for t in m if t is not None]
    if not shapes:
        raise ValueError("map has no non-None entries")
    return shapes[0]


class _TileGrid:
    """Tiles of `tile_shape` over a (ny, nx) map, numbered row by row; the
    last row and column may be short."""

    def __init__(self, shape, tile_shape):
        self.shape = tuple(int(s) for s in shape[-2:])
        self.tile_shape = tile_shape
        self.super_shape = tuple(-(-s // t) for s, t in zip(self.shape, tile_shape))
        self.tile_count = self.super_shape[0] * self.super_shape[1]

    def tile_rowcol(self, tile):
        if tile >= self.tile_count:
            raise ValueError("Request for tile %d is out of bounds for super_shape=%s"
                             % (tile, self.super_shape))
        return divmod(tile, self.super_shape[1])

    def tile_offset(self, tile):
        return tuple(rc * t for rc, t in zip(self.tile_rowcol(tile), self.tile_shape))

    def tile_dims(self, tile):
        return tuple(min(t, s - o) for t, s, o in
                     zip(self.tile_shape, self.shape, self.tile_offset(tile)))


def celestial_to_native(wcs):
    """Rotation taking celestial coordinates to the native spherical
    coordinates of a FITS celestial projection whose reference point
    (CRVAL = (alpha0, delta0)) sits either on the native equator at
    (phi0, theta0) = (0, 0) (cylindrical: CAR, CEA) or at the native pole,
    theta0 = 90 (zenithal: TAN, ZEA, ARC, SIN), with LONPOLE 180 (or 0 for
    a cylindrical map south of the equator): R_z(-alpha0) first, then the
    tilt that brings delta0 to the native equator or pole (and for
    zenithal maps the half turn about the pole that puts LONPOLE at 180).
    python/proj/wcs.py:526-548."""
    w = wcs.wcs
    alpha0, delta0 = (float(v) for v in w.crval)
    spin = quat.euler(2, -alpha0 * quat.DEG)
    ref = (float(w.phi0), float(w.theta0))
    if ref == (0., 0.):
        if not ((delta0 >= 0 and w.lonpole == 180.0) or (delta0 <= 0 and w.lonpole == 0.0)):
            raise ValueError("cylindrical WCS with LONPOLE %g at delta0 %g" % (w.lonpole, delta0))
        return quat.euler(1, delta0 * quat.DEG) * spin
    if ref == (0., 90.):
        if w.lonpole != 180.0:
            raise ValueError("zenithal WCS with LONPOLE %g" % w.lonpole)
        return quat.euler(2, np.pi) * quat.euler(1, (delta0 - 90) * quat.DEG) * spin
    raise ValueError('Unimplemented NSC reference (phi0,theta0)=(%.2f,%.2f)' % ref)


class _Projector:
    """What both Projectionists share: the ProjEng lookup, the cached
    native-frame boresight and the map operations."""

    proj_name = None
    interpol = INTERPOLS[0]
    active_tiles = None
    _map_ndim = None          # dimensions of a whole map: (comp, pixel axes...)

    def __init__(self):
        self._native_cache = (None, None)

    # -- engines --------------------------------------------------------------
    def get_ProjEng(self, comps='TQU', proj_name=None, get=True, instance=True,
                    interpol=None):
        """The ProjEng (class name with get=False, class with
        instance=False) for this geometry and components."""
        name = engine_class_name(proj_name or self.proj_name, comps, bool(self.tiling),
                                 interpol or self.interpol)
        if not get:
            return name
        cls = getattr(_engines(), name, None)
        if cls is None:
            raise ValueError('There is no projector implemented for pixelization "%s", '
                             'components "%s" (tried "%s").'
                             % (proj_name or self.proj_name, comps, name))
        return cls(self._get_pixelizor_args()) if instance else cls

    def _cache_q_fp_to_native(self, q_fp_to_celestial):
        """q_celestial_to_native * Q, computed once per boresight object."""
        held, q_native = self._native_cache
        if held is not q_fp_to_celestial:
            from .coords import _on_device
            if _on_device(q_fp_to_celestial):
                from .. import sightline
                q_native = sightline.left_multiply(self.q_celestial_to_native,
                                                   q_fp_to_celestial)
            else:
                q_native = self.q_celestial_to_native * q_fp_to_celestial
            self._native_cache = (q_fp_to_celestial, q_native)
        return q_native

    def _run(self, comps, method, assembly, *extra, native=True, proj_name=None,
             responses=False):
        """One ProjEng call: method(q, detector quats, [responses,] *extra)."""
        eng = self.get_ProjEng(comps, proj_name=proj_name)
        q = self._cache_q_fp_to_native(assembly.Q) if native else assembly.Q
        fp = assembly.fplane
        lead = (q, fp.quats, fp.resps) if responses else (q, fp.quats)
        return getattr(eng, method)(*lead, *extra)

    def _comps_of(self, shape):
        if len(shape) != self._map_ndim:
            raise ValueError('Cannot guess components based on map with %i!=%i dimensions!'
                             % (len(shape), self._map_ndim))
        if shape[0] not in _COMPS_BY_COUNT:
            raise ValueError('No default components for ncomp=%i; set comps=... explicitly.'
                             % shape[0])
        return _COMPS_BY_COUNT[shape[0]]

    # -- pointing-only products ---------------------------------------------------
    def get_pixels(self, assembly):
        return self._run('TQU', 'pixels', assembly, None)

    def get_pointing_matrix(self, assembly):
        return self._run('TQU', 'pointing_matrix', assembly, None, None, responses=True)

    def get_coords(self, assembly, use_native=False, output=None):
        """Celestial (use_native: native) lon, lat, cos and sin of the
        position angle of every detector and sample."""
        return self._run('TQU', 'coords', assembly, output, native=use_native,
                         proj_name='CAR')

    def get_planar(self, assembly, output=None):
        """Projection-plane coordinates of every detector and sample."""
        return self._run('TQU', 'coords', assembly, output)

    def zeros(self, super_shape):
        return self.get_ProjEng('T').zeros(super_shape)

    # -- maps ------------------------------------------------------------------------
    def to_map(self, signal, assembly, output=None, det_weights=None, threads=None,
               comps=None):
        """Accumulates signal into a map (output, or a new map of comps)."""
        if output is None and comps is None:
            raise ValueError("Provide an output map or specify component of "
                             "interest (e.g. comps='TQU').")
        comps = comps or self._comps_of(_first_tile_shape(output))
        eng = self.get_ProjEng(comps)
        fp = assembly.fplane
        return eng.to_map(output, self._cache_q_fp_to_native(assembly.Q), fp.quats, fp.resps,
                          signal, det_weights, threads)

    def to_weights(self, assembly, output=None, det_weights=None, threads=None, comps=None):
        """Accumulates the pointing weights (ncomp x ncomp per pixel)."""
        if output is None and comps is None:
            raise ValueError("Provide an output map or specify component of "
                             "interest (e.g. comps='TQU').")
        if comps is None:
            shape = _first_tile_shape(output)
            if shape[0] != shape[1]:
                raise ValueError("weight map must be (ncomp, ncomp, ...); got %s" % (shape,))
            comps = self._comps_of(shape[1:])
        eng = self.get_ProjEng(comps)
        fp = assembly.fplane
        return eng.to_weight_map(output, self._cache_q_fp_to_native(assembly.Q), fp.quats,
                                 fp.resps, det_weights, threads)

    def from_map(self, src_map, assembly, signal=None, comps=None):
        """Signal from a map (added into `signal` when given)."""
        src_map = self._with_comp_axis(src_map)
        comps = comps or self._comps_of(_first_tile_shape(src_map))
        eng = self.get_ProjEng(comps)
        fp = assembly.fplane
        return eng.from_map(src_map, self._cache_q_fp_to_native(assembly.Q), fp.quats,
                            fp.resps, signal)

    def _with_comp_axis(self, m):
        return m

    # -- thread assignment -------------------------------------------------------------
    def _check_method(self, method):
        if method not in THREAD_ASSIGNMENT_METHODS:
            raise ValueError('No thread assignment method "%s"; expected one of %s'
                             % (method, THREAD_ASSIGNMENT_METHODS))

    def assign_threads(self, assembly, method='domdir', n_threads=None):
        """thread_intervals for to_map / to_weights: stripes of the map
        ('simple'; 'domdir' gives the same kind of pixel-disjoint bands) or
        groups of tiles ('tiles', which also sets active_tiles)."""
        self._check_method(method)
        n = mapthreads.get_num_threads(n_threads)
        if method == 'tiles':
            info = self.get_active_tiles(assembly, assign=n)
            self.active_tiles = info['active_tiles']
            return info['group_ranges']
        return wrap_ivals(self._run('T', 'pixel_ranges', assembly, None, n))

    def assign_threads_from_map(self, assembly, tmap, n_threads=None):
        """thread_intervals from a map of thread indices."""
        n = mapthreads.get_num_threads(n_threads)
        return wrap_ivals(self._run('T', 'pixel_ranges', assembly, tmap, n))

    def get_active_tiles(self, assembly, assign=False):
        """Tiles the assembly hits and their hit counts; with assign = n (or
        True: the host thread count), also n groups of tiles of balanced
        hits and their sample ranges."""
        if self.tiling is None:
            raise RuntimeError("This Projectionist not set up for Tiled maps.")
        eng = self.get_ProjEng('T')
        q = self._cache_q_fp_to_native(assembly.Q)
        hits = np.asarray(eng.tile_hits(q, assembly.fplane.quats))
        tiles = np.flatnonzero(hits)
        info = {'active_tiles': list(tiles), 'hit_counts': list(hits[tiles])}
        if assign is True:
            assign = _engines().useful_info()['omp_num_threads']
        if assign:
            groups = lpt_groups(hits[tiles], tiles, int(assign))
            info['group_tiles'] = groups
            info['group_ranges'] = wrap_ivals(eng.tile_ranges(q, assembly.fplane.quats, groups))
        return info


class _FlatGeometry:
    """Pixel grid of a celestial WCS (shared by Projectionist instances)."""

    def __init__(self, shape, wcs):
        lng, lat = wcs.wcs.lng, wcs.wcs.lat
        nd = len(shape)
        # naxis in WCS axis order (x = longitude axis first).
        self.naxis = np.array([shape[nd - 1 - lng], shape[nd - 1 - lat]], dtype=int)
        cel = wcs.celestial
        codes = {c[-3:] for c in cel.wcs.ctype}
        if len(codes) != 1:
            raise ValueError("WCS axes have different projections: %s" % sorted(codes))
        self.wcs = cel
        self.proj_name = codes.pop()
        self.cdelt = np.array(cel.wcs.cdelt) * quat.DEG
        self.crpix = np.array(cel.wcs.crpix)


class Projectionist(_Projector):
    """Projector for rectangular-pixel maps (CAR, CEA, TAN, ZEA, ARC, SIN),
    untiled or tiled."""

    _map_ndim = 3

    get_q = staticmethod(celestial_to_native)

    def __init__(self):
        super().__init__()
        self.tile_shape = None
        self.active_tiles = None
        self.wcs = None
        self.proj_name = None
        self.q_celestial_to_native = None
        self.interpol = INTERPOLS[0]
        self.naxis = np.array([0, 0])
        self.cdelt = np.array([0., 0.])
        self.crpix = np.array([0., 0.])

    @property
    def tiling(self):
        if self.tile_shape is None:
            return None
        return _TileGrid(self.naxis[::-1], self.tile_shape)

    @classmethod
    def for_geom(cls, shape, wcs, interpol=None):
        """Projector for a map of `shape` (..., ny, nx) on `wcs`."""
        g = _FlatGeometry(shape, wcs)
        self = cls()
        self.naxis, self.wcs, self.proj_name = g.naxis, g.wcs, g.proj_name
        self.cdelt, self.crpix = g.cdelt, g.crpix
        self.q_celestial_to_native = celestial_to_native(g.wcs)
        self.interpol = interpol or INTERPOLS[0]
        return self

    @classmethod
    def for_map(cls, emap, wcs=None, interpol=None):
        return cls.for_geom(emap.shape, emap.wcs if wcs is None else wcs, interpol=interpol)

    @classmethod
    def for_source_at(cls, alpha0, delta0, gamma0=0., proj_name='TAN'):
        """Projector whose native pole is at (alpha0, delta0) (degrees)."""
        if gamma0 != 0.:
            raise ValueError("only gamma0 = 0 is supported")
        self = cls()
        self.proj_name = proj_name
        self.q_celestial_to_native = (quat.euler(2, np.pi) *
                                      quat.euler(1, (delta0 - 90) * quat.DEG) *
                                      quat.euler(2, -alpha0 * quat.DEG))
        return self

    @classmethod
    def for_tiled(cls, shape, wcs, tile_shape, active_tiles=True, interpol=None):
        """for_geom with the map cut into tiles of tile_shape; active_tiles:
        True (every tile), False/None (to be found), or a list."""
        self = cls.for_geom(shape, wcs, interpol=interpol)
        self.tile_shape = np.array(tile_shape, 'int')
        if active_tiles is True:
            self.active_tiles = list(range(self.tiling.tile_count))
        elif active_tiles is False or active_tiles is None:
            self.active_tiles = None
        else:
            self.active_tiles = active_tiles
        return self

    def _with_comp_axis(self, m):
        if not isinstance(m, list) and m.ndim == 2:
            return m[None]
        return m

    def _get_pixelizor_args(self):
        """(ny, nx, cdelt_y, cdelt_x, crpix_y, crpix_x[, tile_y, tile_x
        [, active_tiles]]): the ProjEng constructor argument."""
        nx, ny = (int(v) for v in self.naxis)
        dx, dy = (float(v) for v in self.cdelt)
        px, py = (float(v) for v in self.crpix)
        args = (ny, nx, dy, dx, py, px)
        if self.tiling:
            args += tuple(int(v) for v in self.tile_shape)
            if self.active_tiles is not None:
                args += (self.active_tiles,)
        return args


class ProjectionistHealpix(_Projector):
    """Projector for HEALPix maps (NEST or RING; tiled maps NEST only).
    The native frame is the celestial frame."""

    _map_ndim = 2

    def __init__(self):
        super().__init__()
        self.active_tiles = None
        self.proj_name = None
        self.q_celestial_to_native = quat.quat(1, 0, 0, 0)
        self.interpol = 'nearest'
        self.tiling = None
        self.nside = None
        self.nside_tile = None
        self.ordering = 'NEST'

    @classmethod
    def for_healpix(cls, nside, nside_tile=None, active_tiles=None, ordering='NEST',
                    interpol=None):
        """Projector for nside; nside_tile (an int, or 'auto' to choose one
        from the hit tiles) makes a tiled map."""
        if interpol not in (None, 'nearest', 'nn'):
            raise NotImplementedError("Only 'nearest' interpolation is supported for Healpix")
        if ordering not in ('NEST', 'RING'):
            raise ValueError("ordering %s should be 'NEST' or 'RING'" % ordering)
        if ordering == 'RING' and nside_tile is not None:
            raise NotImplementedError("'RING' not supported for tiled maps")
        self = cls()
        self.proj_name = 'HP'
        self.nside = nside
        self.ordering = ordering
        self.active_tiles = active_tiles
        if nside_tile is not None:
            self.nside_tile = nside_tile
            self.tiling = True
        return self

    def compute_nside_tile(self, assembly, nActivePerThread=5, nThreads=None):
        """Resolves nside_tile='auto': from the fraction of the sky the
        assembly hits at nside_tile 4, the power of two giving about
        nActivePerThread hit tiles per thread (at most nside)."""
        if self.nside_tile != 'auto':
            return self.nside_tile
        self.nside_tile = min(4, self.nside)
        n_hit = len(self.get_active_tiles(assembly)['active_tiles'])
        fsky = n_hit / (12 * self.nside_tile ** 2)
        if nThreads is None:
            nThreads = _engines().useful_info()['omp_num_threads']
        want = nActivePerThread * nThreads / (12 * fsky)
        self.nside_tile = min(int(2 ** np.ceil(0.5 * np.log2(want))), self.nside)
        return self.nside_tile

    def get_active_tiles(self, assembly, assign=False):
        self.compute_nside_tile(assembly)
        return super().get_active_tiles(assembly, assign)

    def get_coords(self, assembly, use_native=False, output=None):
        return self._run('TQU', 'coords', assembly, output, native=use_native)

    def _with_comp_axis(self, m):
        if self.nside_tile is None:
            return m[None] if m.ndim == 1 else m
        if not isinstance(m, list):
            raise TypeError("Expected list for tiled map; src_map is %s" % type(m))
        if len(_first_tile_shape(m)) == 1:
            for i, t in enumerate(m):
                if t is not None:
                    m[i] = t[None]
        return m

    def _check_method(self, method):
        if method in THREAD_ASSIGNMENT_METHODS and method not in THREAD_ASSIGNMENT_METHODS_HP:
            raise ValueError('Thread assignment method "%s" not supported for '
                             'ProjectionistHealpix. Expected one of %s.'
                             % (method, THREAD_ASSIGNMENT_METHODS_HP))
        super()._check_method(method)

    def assign_threads(self, assembly, method=None, n_threads=None):
        if method is None:
            method = 'tiles' if self.nside_tile is not None else 'simple'
        return super().assign_threads(assembly, method, n_threads)

    def _get_pixelizor_args(self):
        """(nside, nest, nside_tile, active_tiles)."""
        tiles = None if self.active_tiles is None else [int(t) for t in self.active_tiles]
        nt = None if self.nside_tile is None else int(self.nside_tile)
        return (int(self.nside), int(self.ordering == 'NEST'), nt, tiles)
