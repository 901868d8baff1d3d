"""Pointing inputs of the so3g.proj API (python/proj/coords.py): sight
lines (boresight quaternions), focal planes (detector offsets and (T, P)
responses) and assemblies (a sight line with a focal plane attached).

Sight lines are built from rotations composed right to left onto the
boresight's "up" axis: roll about it, then the elevation tilt, then the
azimuth turn (horizon frame), and for naive_az_el the site's latitude and
the Earth rotation angle (celestial frame, no precession, nutation,
aberration or refraction).  The qpoint-based ``az_el`` needs the qpoint
package, which is not part of this library.

Sight lines given CUDA tensors are built on the GPU (so3g_gb300.sightline),
by the same sequence of products.
"""
import numpy as np

from . import quat

DEG = np.pi / 180.

# Earth rotation angle at unix time t (days J since the J2000.0 epoch, 12h
# UT 2000-01-01): ERA = 2 pi (0.7790572732640 + 1.00273781191135448 J),
# stored as the coefficients of polyval(ERA_POLY, J).
ERA_EPOCH = 946684800 + 3600 * 12
ERA_POLY = np.array([6.300387486754831, 4.894961212823756])


class EarthlySite:
    """An observing site: longitude (deg E), latitude (deg N), elevation
    (m) and, optionally, typical weather."""

    def __init__(self, lon, lat, elev, typical_weather=None):
        self.lon, self.lat, self.elev = lon, lat, elev
        self.typical_weather = typical_weather


def _dms(d, m, s):
    return d + m / 60. + s / 3600.


# Site coordinates (data): the ACT site and the Simons Observatory LAT and
# SATs in the Atacama.
SITES = {
    'act': EarthlySite(-67.7876, -22.9585, 5188.),
    'so_lat': EarthlySite(-_dms(67, 47, 15.68), -_dms(22, 57, 39.47), 5188.),
    'so_sat1': EarthlySite(-_dms(67, 47, 18.11), -_dms(22, 57, 36.38), 5188.),
    'so_sat2': EarthlySite(-_dms(67, 47, 17.28), -_dms(22, 57, 36.35), 5188.),
    'so_sat3': EarthlySite(-_dms(67, 47, 16.53), -_dms(22, 57, 35.97), 5188.),
}
SITES['so'] = SITES['so_lat']
SITES['_default'] = SITES['so']
DEFAULT_SITE = 'so'


def _on_device(*xs):
    """True if any argument is a CUDA torch tensor (torch is looked up only
    if already imported)."""
    import sys
    torch = sys.modules.get("torch")
    return torch is not None and any(isinstance(x, torch.Tensor) and x.is_cuda for x in xs)


def _site(site):
    if site is None:
        site = DEFAULT_SITE
    if isinstance(site, EarthlySite):
        return site
    found = SITES.get(site)
    if found is None:
        raise ValueError("Could not decode %s as a Site." % site)
    return found


def _horizon(az, el, roll):
    """Horizon-frame boresight: azimuth turn, elevation tilt, roll."""
    return quat.euler(2, -az) * quat.euler(1, np.pi / 2 - el) * quat.euler(2, roll)


class CelestialSightLine:
    """A vector of boresight quaternions, ``Q`` (focal plane -> celestial)."""

    decode_site = staticmethod(_site)

    @classmethod
    def _of(cls, Q):
        self = cls()
        self.Q = Q
        return self

    @classmethod
    def naive_az_el(cls, t, az, el, roll=0., site=None, weather=None):
        """Boresight at unix times t from horizon az, el, roll (radians):
        the horizon frame turned by the site's latitude and the Earth
        rotation angle only."""
        site = _site(site)
        if _on_device(t, az, el, roll):
            from .. import sightline
            return cls._of(sightline.boresight("naive", t, az, el, roll, site=site))
        lst = np.polyval(ERA_POLY, (np.asarray(t) - ERA_EPOCH) / 86400) + site.lon * DEG
        to_celestial = (quat.euler(2, lst) * quat.euler(1, np.pi / 2 - site.lat * DEG) *
                        quat.euler(2, np.pi))
        # Composed left to right, as the device kernel does.
        Q = (to_celestial * quat.euler(2, -np.asarray(az)) *
             quat.euler(1, np.pi / 2 - np.asarray(el)) * quat.euler(2, roll))
        return cls._of(Q)

    @classmethod
    def az_el(cls, t, az, el, roll=None, site=None, weather=None, **kwargs):
        try:
            import qpoint  # noqa: F401
        except ImportError:
            raise ImportError("CelestialSightLine.az_el needs the qpoint package; use "
                              "naive_az_el or for_horizon instead") from None
        raise NotImplementedError("qpoint-based pointing is not part of so3g_gb300")

    @classmethod
    def for_lonlat(cls, lon, lat, psi=0):
        """Boresight pointing at (lon, lat) with position angle psi."""
        return cls._of(quat.euler(2, lon) * quat.euler(1, np.pi / 2 - np.asarray(lat)) *
                       quat.euler(2, psi))

    @classmethod
    def for_horizon(cls, t, az, el, roll=None, site=None, weather=None):
        """The horizon frame itself taken as the celestial frame."""
        if _on_device(az, el, roll):
            from .. import sightline
            return cls._of(sightline.boresight("horizon", t, az, el, roll))
        return cls._of(_horizon(np.asarray(az), np.asarray(el),
                                0. if roll is None else np.asarray(roll)))

    def coords(self, fplane=None, output=None):
        """(lon, lat, cos psi, sin psi) of each detector of fplane (default:
        the boresight alone, without the detector axis) at each time."""
        import so3g_gb300
        eng = so3g_gb300.ProjEng_CAR_TQU_NonTiled((1, 1, 1., 1., 1., 1.))
        if fplane is not None:
            return eng.coords(self.Q, fplane.quats, output)
        out = eng.coords(self.Q, FocalPlane.boresight().quats,
                         None if output is None else output[None])
        return out[0]


class FocalPlane:
    """Detector offset quaternions (``quats``, (n_det, 4) G3VectorQuat) and
    (T, P) responses (``resps``, float32 (n_det, 2)), optionally named."""

    def __init__(self, quats=None, resps=None, dets=None):
        q = quats if isinstance(quats, quat.G3VectorQuat) else \
            quat.G3VectorQuat(np.asarray([] if quats is None else quats,
                                         dtype=np.float64).reshape(-1, 4))
        r = np.ones((len(q), 2), np.float32)
        if resps is not None:
            r[:] = resps
        for what, arr in (("quaternions", np.asarray(q)), ("responses", r)):
            if not np.all(np.isfinite(arr)):
                raise ValueError("nan/inf values in detector %s" % what)
        self.quats, self.resps = q, r
        self._dets = [] if dets is None else list(dets)

    @classmethod
    def boresight(cls):
        """A single detector on the boresight."""
        return cls(quats=[[1., 0., 0., 0.]])

    @classmethod
    def from_xieta(cls, xi, eta, gamma=0, T=1, P=1, Q=1, U=0, hwp=False, dets=None):
        """Detectors at focal-plane (xi, eta) with polarisation angle gamma
        and responses T, P; a polarisation given as (Q, U) turns gamma by
        arctan2(U, Q)/2 and scales P by |(Q, U)|; hwp reverses gamma."""
        gamma = gamma + np.arctan2(U, Q) / 2
        P = P * np.hypot(Q, U)
        if hwp:
            gamma = -gamma
        xi, eta, gamma, T, P, _ = np.broadcast_arrays(xi, eta, gamma, T, P, [0])
        resps = np.stack([np.asarray(T, float), np.asarray(P, float)], axis=1)
        return cls(quat.rotation_xieta(xi, eta, gamma), resps=resps, dets=dets)

    def coeffs(self):
        return np.array(self.quats, dtype=np.float64)

    @property
    def ndet(self):
        return len(self.quats)

    def __len__(self):
        return self.ndet

    def __getitem__(self, sel):
        if isinstance(sel, str):
            return self.quats[self._dets.index(sel)]
        return FocalPlane(quats=self.coeffs()[sel], resps=self.resps[sel])

    def items(self):
        return zip(self.quats, self.resps)

    def __repr__(self):
        return "FocalPlane(quats=%r,resps=%r)" % (self.coeffs(), self.resps)


class Assembly:
    """A sight line (``Q``) with a rigidly attached focal plane (``fplane``)."""

    def __init__(self, collapse=False):
        self.collapse = collapse

    @classmethod
    def attach(cls, sight_line, fplane):
        self = cls()
        self.Q = sight_line if isinstance(sight_line, quat.G3VectorQuat) else sight_line.Q
        self.fplane = fplane
        return self

    @classmethod
    def for_boresight(cls, sight_line):
        """The sight line with one detector on the boresight; collapse=True."""
        self = cls(collapse=True)
        self.Q = sight_line.Q
        self.fplane = FocalPlane.boresight()
        return self

    @property
    def dets(self):
        return self.fplane
