"""Projectionist front-ends of so3g.proj.wcs (python/proj/wcs.py), over the
GB300 ProjEng classes.

Quaternion naming as in the reference: assembly.Q takes focal-plane to
celestial coordinates, the detector quaternions take detector to focal
plane, and ``q_celestial_to_native`` takes celestial to the native
spherical coordinates of the projection.  The Projectionist caches
``q_native = q_celestial_to_native * assembly.Q`` and passes it, with the
detector quaternions, to the ProjEng methods.

The ``threads`` argument of the projection methods is accepted in every
form the reference accepts.  The GPU kernels need no pixel-disjoint thread
domains (they accumulate with atomics), so a thread assignment only
selects samples; any of the assignment methods gives the same maps.
"""
import numpy as np

from . import quat
from . import mapthreads
from ..ranges import RangesMatrix, RangesInt32, wrap_ivals  # noqa: F401

Ranges = RangesInt32

#: Valid settings for "interpol"; the first entry is the default.
INTERPOLS = ['nearest', 'bilinear']

THREAD_ASSIGNMENT_METHODS = ['simple', 'domdir', 'tiles']
THREAD_ASSIGNMENT_METHODS_HP = ['simple', 'tiles']


def _so3g():
    import so3g_gb300
    return so3g_gb300


class _ProjectionistBase:
    """Shared logic of Projectionist and ProjectionistHealpix
    (python/proj/wcs.py:41-476)."""

    def __init__(self):
        raise NotImplementedError("Use child class Projectionist or ProjectionistHealpix")

    def _get_pixelizor_args(self):
        raise NotImplementedError("Use child class Projectionist or ProjectionistHealpix")

    def get_ProjEng(self, comps='TQU', proj_name=None, get=True, instance=True, interpol=None):
        """The ProjEng object for this geometry (python/proj/wcs.py:108-138)."""
        if proj_name is None:
            proj_name = self.proj_name
        tile_suffix = 'Tiled' if self.tiling else 'NonTiled'
        if interpol is None:
            interpol = self.interpol
        if interpol in ["nn", "nearest"]:
            interpol_suffix = ""
        elif interpol in ["lin", "bilinear"]:
            interpol_suffix = "_Bilinear"
        else:
            raise ValueError("ProjEng interpol '%s' not recognized" % str(interpol))
        projeng_name = f'ProjEng_{proj_name}_{comps}_{tile_suffix}{interpol_suffix}'
        if not get:
            return projeng_name
        try:
            projeng_cls = getattr(_so3g(), projeng_name)
        except AttributeError:
            raise ValueError(f'There is no projector implemented for '
                             f'pixelization "{proj_name}", components '
                             f'"{comps}" (tried "{projeng_name}").') from None
        if not instance:
            return projeng_cls
        return projeng_cls(self._get_pixelizor_args())

    def _cache_q_fp_to_native(self, q_fp_to_celestial):
        if q_fp_to_celestial is not self._q_fp_to_celestial:
            from .coords import _on_device
            if _on_device(q_fp_to_celestial):
                # A boresight held on the device: the product runs there.
                from .. import sightline
                self._q_fp_to_native = sightline.left_multiply(self.q_celestial_to_native,
                                                               q_fp_to_celestial)
            else:
                self._q_fp_to_native = self.q_celestial_to_native * q_fp_to_celestial
            self._q_fp_to_celestial = q_fp_to_celestial
        return self._q_fp_to_native

    def _guess_comps(self, map_shape):
        if map_shape[0] == 1:
            return 'T'
        elif map_shape[0] == 2:
            return 'QU'
        elif map_shape[0] == 3:
            return 'TQU'
        raise ValueError('No default components for ncomp=%i; '
                         'set comps=... explicitly.' % map_shape[0])

    def _get_map_shape(self, imap):
        if isinstance(imap, list):
            for tile in imap:
                if tile is not None:
                    return tuple(tile.shape)
            raise ValueError("map has no non-None entries")
        return tuple(imap.shape)

    def get_pixels(self, assembly):
        projeng = self.get_ProjEng('TQU')
        q_native = self._cache_q_fp_to_native(assembly.Q)
        return projeng.pixels(q_native, assembly.fplane.quats, None)

    def get_pointing_matrix(self, assembly):
        projeng = self.get_ProjEng('TQU')
        q_native = self._cache_q_fp_to_native(assembly.Q)
        return projeng.pointing_matrix(q_native, assembly.fplane.quats,
                                       assembly.fplane.resps, None, None)

    def get_coords(self, assembly, use_native=False, output=None):
        projeng = self.get_ProjEng('TQU', 'CAR')
        if use_native:
            q_native = self._cache_q_fp_to_native(assembly.Q)
        else:
            q_native = assembly.Q
        return projeng.coords(q_native, assembly.fplane.quats, output)

    def get_planar(self, assembly, output=None):
        q_native = self._cache_q_fp_to_native(assembly.Q)
        projeng = self.get_ProjEng('TQU')
        return projeng.coords(q_native, assembly.fplane.quats, output)

    def zeros(self, super_shape):
        projeng = self.get_ProjEng('T')
        return projeng.zeros(super_shape)

    def to_map(self, signal, assembly, output=None, det_weights=None, threads=None,
               comps=None):
        """Project signal into a map (python/proj/wcs.py:255-277)."""
        if output is None and comps is None:
            raise ValueError("Provide an output map or specify component of "
                             "interest (e.g. comps='TQU').")
        if comps is None:
            comps = self._guess_comps(self._get_map_shape(output))
        projeng = self.get_ProjEng(comps)
        q_native = self._cache_q_fp_to_native(assembly.Q)
        return projeng.to_map(output, q_native, assembly.fplane.quats,
                              assembly.fplane.resps, signal, det_weights, threads)

    def to_weights(self, assembly, output=None, det_weights=None, threads=None, comps=None):
        """Project pointing into a weights map (python/proj/wcs.py:279-303)."""
        if output is None and comps is None:
            raise ValueError("Provide an output map or specify component of "
                             "interest (e.g. comps='TQU').")
        if comps is None:
            shape = self._get_map_shape(output)
            assert shape[0] == shape[1]
            comps = self._guess_comps(shape[1:])
        projeng = self.get_ProjEng(comps)
        q_native = self._cache_q_fp_to_native(assembly.Q)
        return projeng.to_weight_map(output, q_native, assembly.fplane.quats,
                                     assembly.fplane.resps, det_weights, threads)

    def from_map(self, src_map, assembly, signal=None, comps=None):
        """De-project from a map (python/proj/wcs.py:305-323)."""
        if comps is None:
            comps = self._guess_comps(self._get_map_shape(src_map))
        projeng = self.get_ProjEng(comps)
        q_native = self._cache_q_fp_to_native(assembly.Q)
        return projeng.from_map(src_map, q_native, assembly.fplane.quats,
                                assembly.fplane.resps, signal)

    def assign_threads(self, assembly, method='domdir', n_threads=None):
        """A thread assignment (python/proj/wcs.py:325-386).  'domdir' builds
        the same kind of pixel-disjoint bands as 'simple' (stripes of the
        map); the GPU kernels do not depend on the assignment."""
        if method not in THREAD_ASSIGNMENT_METHODS:
            raise ValueError(f'No thread assignment method "{method}"; '
                             f'expected one of {THREAD_ASSIGNMENT_METHODS}')
        n_threads = mapthreads.get_num_threads(n_threads)
        if method in ('simple', 'domdir'):
            projeng = self.get_ProjEng('T')
            q_native = self._cache_q_fp_to_native(assembly.Q)
            omp_ivals = projeng.pixel_ranges(q_native, assembly.fplane.quats, None, n_threads)
            return wrap_ivals(omp_ivals)
        tile_info = self.get_active_tiles(assembly, assign=n_threads)
        self.active_tiles = tile_info['active_tiles']
        return tile_info['group_ranges']

    def assign_threads_from_map(self, assembly, tmap, n_threads=None):
        projeng = self.get_ProjEng('T')
        q_native = self._cache_q_fp_to_native(assembly.Q)
        n_threads = mapthreads.get_num_threads(n_threads)
        omp_ivals = projeng.pixel_ranges(q_native, assembly.fplane.quats, tmap, n_threads)
        return wrap_ivals(omp_ivals)

    def get_active_tiles(self, assembly, assign=False):
        """Tiles hit by an assembly, optionally grouped into n threads
        (python/proj/wcs.py:408-474)."""
        if self.tiling is None:
            raise RuntimeError("This Projectionist not set up for Tiled maps.")
        projeng = self.get_ProjEng('T')
        q_native = self._cache_q_fp_to_native(assembly.Q)
        hits = np.array(projeng.tile_hits(q_native, assembly.fplane.quats))
        tiles = np.nonzero(hits)[0]
        hits = hits[tiles]
        if assign is True:
            assign = _so3g().useful_info()['omp_num_threads']
        if assign > 0:
            group_n = np.array([0 for g in range(assign)])
            group_tiles = [[] for _ in group_n]
            cands = sorted(list(zip(hits, tiles)), reverse=True)
            for _n, _t in cands:
                idx = group_n.argmin()
                group_n[idx] += _n
                group_tiles[idx].append(_t)
            R = projeng.tile_ranges(q_native, assembly.fplane.quats, group_tiles)
            R = wrap_ivals(R)
            return {'active_tiles': list(tiles), 'hit_counts': list(hits),
                    'group_ranges': R, 'group_tiles': group_tiles}
        return {'active_tiles': list(tiles), 'hit_counts': list(hits)}


class Projectionist(_ProjectionistBase):
    """Rectangular-pixel Projectionist (python/proj/wcs.py:478-701)."""

    @staticmethod
    def get_q(wcs):
        """Rotation from celestial to native spherical coordinates
        (python/proj/wcs.py:526-548)."""
        alpha0, delta0 = wcs.wcs.crval
        if wcs.wcs.phi0 == 0. and wcs.wcs.theta0 == 0.:
            assert ((delta0 >= 0 and wcs.wcs.lonpole == 180.0) or
                    (delta0 <= 0 and wcs.wcs.lonpole == 0.0))
            Q = (quat.euler(1, delta0 * quat.DEG) * quat.euler(2, -alpha0 * quat.DEG))
        elif wcs.wcs.phi0 == 0. and wcs.wcs.theta0 == 90.:
            assert wcs.wcs.lonpole == 180.0
            Q = (quat.euler(2, np.pi) * quat.euler(1, (delta0 - 90) * quat.DEG) *
                 quat.euler(2, -alpha0 * quat.DEG))
        else:
            raise ValueError(f'Unimplemented NSC reference (phi0,theta0)='
                             f'({wcs.wcs.phi0:.2f},{wcs.wcs.theta0:.2f})')
        return Q

    def __init__(self):
        self._q_fp_to_native = None
        self._q_fp_to_celestial = None
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
        return _Tiling(self.naxis[::-1], self.tile_shape)

    @classmethod
    def for_geom(cls, shape, wcs, interpol=None):
        self = cls()
        ax1, ax2 = wcs.wcs.lng, wcs.wcs.lat
        ndim = len(shape)
        self.naxis = np.array([shape[ndim - ax1 - 1], shape[ndim - ax2 - 1]], dtype=int)
        wcs = wcs.celestial
        self.wcs = wcs
        proj = [c[-3:] for c in wcs.wcs.ctype]
        assert proj[0] == proj[1]
        self.proj_name = proj[0]
        self.q_celestial_to_native = self.get_q(wcs)
        self.cdelt = np.array(wcs.wcs.cdelt) * quat.DEG
        self.crpix = np.array(wcs.wcs.crpix)
        self.interpol = INTERPOLS[0] if interpol is None else interpol
        return self

    @classmethod
    def for_map(cls, emap, wcs=None, interpol=None):
        if wcs is None:
            wcs = emap.wcs
        return cls.for_geom(emap.shape, wcs, interpol=interpol)

    @classmethod
    def for_source_at(cls, alpha0, delta0, gamma0=0., proj_name='TAN'):
        self = cls()
        self.proj_name = proj_name
        assert gamma0 == 0.
        self.q_celestial_to_native = (quat.euler(2, np.pi) *
                                      quat.euler(1, (delta0 - 90) * quat.DEG) *
                                      quat.euler(2, -alpha0 * quat.DEG))
        return self

    @classmethod
    def for_tiled(cls, shape, wcs, tile_shape, active_tiles=True, interpol=None):
        self = cls.for_geom(shape, wcs, interpol=interpol)
        self.tile_shape = np.array(tile_shape, 'int')
        if active_tiles is True:
            self.active_tiles = list(range(self.tiling.tile_count))
        elif active_tiles in [False, None]:
            self.active_tiles = None
        else:
            self.active_tiles = active_tiles
        return self

    def from_map(self, src_map, assembly, signal=None, comps=None):
        if not isinstance(src_map, list) and src_map.ndim == 2:
            src_map = src_map[None]
        return super().from_map(src_map, assembly, signal, comps)

    def _get_pixelizor_args(self):
        args = (int(self.naxis[1]), int(self.naxis[0]),
                float(self.cdelt[1]), float(self.cdelt[0]),
                float(self.crpix[1]), float(self.crpix[0]))
        if self.tiling:
            args += tuple(map(int, self.tile_shape))
            if self.active_tiles is not None:
                args += (self.active_tiles,)
        return args

    def _guess_comps(self, map_shape):
        if len(map_shape) != 3:
            raise ValueError('Cannot guess components based on '
                             'map with %i!=3 dimensions!' % len(map_shape))
        return super()._guess_comps(map_shape)


class ProjectionistHealpix(_ProjectionistBase):
    """HEALPix Projectionist (python/proj/wcs.py:704-860)."""

    def __init__(self):
        self._q_fp_to_native = None
        self._q_fp_to_celestial = None
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
        self = cls()
        self.proj_name = 'HP'
        self.nside = nside
        self.active_tiles = active_tiles
        if interpol is not None and (interpol not in ['nearest', 'nn']):
            raise NotImplementedError("Only 'nearest' interpolation is supported for Healpix")
        self.interpol = 'nearest'
        self.ordering = ordering
        if ordering not in ['NEST', 'RING']:
            raise ValueError(f"ordering {ordering} should be 'NEST' or 'RING'")
        if nside_tile is not None:
            self.nside_tile = nside_tile
            self.tiling = True
        if ordering == 'RING' and self.nside_tile is not None:
            raise NotImplementedError("'RING' not supported for tiled maps")
        return self

    def compute_nside_tile(self, assembly, nActivePerThread=5, nThreads=None):
        """Pick nside_tile for nside_tile='auto' (python/proj/wcs.py:759-778)."""
        if self.nside_tile == 'auto':
            nside_tile0 = min(4, self.nside)
            self.nside_tile = nside_tile0
            nActive = len(self.get_active_tiles(assembly)['active_tiles'])
            fsky = nActive / (12 * nside_tile0 ** 2)
            if nThreads is None:
                nThreads = _so3g().useful_info()['omp_num_threads']
            self.nside_tile = int(2 ** np.ceil(0.5 * np.log2(nActivePerThread * nThreads /
                                                              (12 * fsky))))
            self.nside_tile = min(self.nside_tile, self.nside)
        return self.nside_tile

    def get_active_tiles(self, assembly, assign=False):
        self.compute_nside_tile(assembly)
        return super().get_active_tiles(assembly, assign)

    def get_coords(self, assembly, use_native=False, output=None):
        projeng = self.get_ProjEng('TQU')
        q_native = self._cache_q_fp_to_native(assembly.Q) if use_native else assembly.Q
        return projeng.coords(q_native, assembly.fplane.quats, output)

    def from_map(self, src_map, assembly, signal=None, comps=None):
        if self.nside_tile is None and src_map.ndim == 1:
            src_map = src_map[None]
        elif self.nside_tile is not None:
            if not isinstance(src_map, list):
                raise TypeError(f"Expected list for tiled map; src_map is {type(src_map)}")
            shape = self._get_map_shape(src_map)
            if len(shape) == 1:
                for itile in range(len(src_map)):
                    if src_map[itile] is not None:
                        src_map[itile] = src_map[itile][None]
        return super().from_map(src_map, assembly, signal, comps)

    def assign_threads(self, assembly, method=None, n_threads=None):
        if method is None:
            method = 'simple' if self.nside_tile is None else 'tiles'
        if (method not in THREAD_ASSIGNMENT_METHODS_HP) and \
                (method in THREAD_ASSIGNMENT_METHODS):
            raise ValueError(f'Thread assignment method "{method}" not supported for '
                             f'ProjectionistHealpix. Expected one of '
                             f'{THREAD_ASSIGNMENT_METHODS_HP}.')
        return super().assign_threads(assembly, method, n_threads)

    def _get_pixelizor_args(self):
        active_tiles = None if self.active_tiles is None else list(map(int, self.active_tiles))
        nside_tile = None if self.nside_tile is None else int(self.nside_tile)
        return (int(self.nside), int(self.ordering == 'NEST'), nside_tile, active_tiles)

    def _guess_comps(self, map_shape):
        if len(map_shape) != 2:
            raise ValueError('Cannot guess components based on '
                             'map with %i!=2 dimensions!' % len(map_shape))
        return super()._guess_comps(map_shape)


class _Tiling:
    """Tile arithmetic of a tiled map (python/proj/wcs.py:863-885)."""

    def __init__(self, shape, tile_shape):
        self.shape = shape[-2:]
        self.tile_shape = tile_shape
        nt0 = int(np.ceil(self.shape[0] / self.tile_shape[0]))
        nt1 = int(np.ceil(self.shape[1] / self.tile_shape[1]))
        self.super_shape = (nt0, nt1)
        self.tile_count = nt0 * nt1

    def tile_dims(self, tile):
        rowcol = self.tile_rowcol(tile)
        return (min(self.shape[0] - rowcol[0] * self.tile_shape[0], self.tile_shape[0]),
                min(self.shape[1] - rowcol[1] * self.tile_shape[1], self.tile_shape[1]))

    def tile_rowcol(self, tile):
        if tile >= self.tile_count:
            raise ValueError(f"Request for tile {tile} is out of bounds for "
                             f"super_shape={self.super_shape}")
        return (tile // self.super_shape[1], tile % self.super_shape[1])

    def tile_offset(self, tile):
        row, col = self.tile_rowcol(tile)
        return row * self.tile_shape[0], col * self.tile_shape[1]
