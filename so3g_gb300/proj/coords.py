"""Pointing inputs of so3g.proj.coords (python/proj/coords.py): sight
lines (boresight quaternions), focal planes (detector offsets and
responses) and assemblies.

The high-precision ``az_el`` (qpoint) constructor needs the qpoint package;
``naive_az_el``, ``for_lonlat`` and ``for_horizon`` are self-contained.
"""
import numpy as np

from . import quat

DEG = np.pi / 180.


class EarthlySite:
    def __init__(self, lon, lat, elev, typical_weather=None):
        """Arguments in degrees E, degrees N, meters above sea level."""
        self.lon, self.lat, self.elev = lon, lat, elev
        self.typical_weather = typical_weather


def _debabyl(deg, arcmin, arcsec):
    return deg + arcmin / 60 + arcsec / 3600


SITES = {
    'act': EarthlySite(-67.7876, -22.9585, 5188.),
    'so_lat': EarthlySite(-_debabyl(67, 47, 15.68), -_debabyl(22, 57, 39.47), 5188.),
    'so_sat1': EarthlySite(-_debabyl(67, 47, 18.11), -_debabyl(22, 57, 36.38), 5188.),
    'so_sat2': EarthlySite(-_debabyl(67, 47, 17.28), -_debabyl(22, 57, 36.35), 5188.),
    'so_sat3': EarthlySite(-_debabyl(67, 47, 16.53), -_debabyl(22, 57, 35.97), 5188.),
}
SITES['so'] = SITES['so_lat']
SITES['_default'] = SITES['so']
DEFAULT_SITE = 'so'

# Naive horizon -> celestial conversion (python/proj/coords.py:63-66).
ERA_EPOCH = 946684800 + 3600 * 12
ERA_POLY = np.array([6.300387486754831, 4.894961212823756])


def _on_device(*xs):
    """True if any argument is a CUDA torch tensor (torch imported only when
    one could be)."""
    import sys
    torch = sys.modules.get("torch")
    return torch is not None and any(isinstance(x, torch.Tensor) and x.is_cuda for x in xs)


class CelestialSightLine:
    """A vector of boresight pointing quaternions, in ``self.Q``."""

    @staticmethod
    def decode_site(site=None):
        if site is None:
            site = DEFAULT_SITE
        if isinstance(site, EarthlySite):
            return site
        if site in SITES:
            return SITES[site]
        raise ValueError("Could not decode %s as a Site." % site)

    @classmethod
    def naive_az_el(cls, t, az, el, roll=0., site=None, weather=None):
        """Horizon (az, el) at unix times t, rotated to celestial with the
        Earth rotation angle only (python/proj/coords.py:99-125)."""
        site = cls.decode_site(site)
        self = cls()
        if _on_device(t, az, el, roll):
            # CUDA tensors in: the boresight is formed on the device.
            from .. import sightline
            self.Q = sightline.boresight("naive", t, az, el, roll, site=site)
            return self
        J = (np.asarray(t) - ERA_EPOCH) / 86400
        era = np.polyval(ERA_POLY, J)
        lst = era + site.lon * DEG
        self.Q = (quat.euler(2, lst) * quat.euler(1, np.pi / 2 - site.lat * DEG) *
                  quat.euler(2, np.pi) * quat.euler(2, -np.asarray(az)) *
                  quat.euler(1, np.pi / 2 - np.asarray(el)) * quat.euler(2, roll))
        return self

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
        """(python/proj/coords.py:171-188)"""
        self = cls()
        self.Q = quat.euler(2, lon) * quat.euler(1, np.pi / 2 - np.asarray(lat)) * \
            quat.euler(2, psi)
        return self

    @classmethod
    def for_horizon(cls, t, az, el, roll=None, site=None, weather=None):
        """Local horizon coordinates taken as "celestial"
        (python/proj/coords.py:190-209)."""
        self = cls()
        if _on_device(az, el, roll):
            # CUDA tensors in: the boresight is formed on the device.
            from .. import sightline
            self.Q = sightline.boresight("horizon", t, az, el, roll)
            return self
        az, el, t = map(np.asarray, [az, el, t])
        roll = 0. if roll is None else np.asarray(roll)
        self.Q = (quat.euler(2, -az) * quat.euler(1, np.pi / 2 - el) * quat.euler(2, roll))
        return self

    def coords(self, fplane=None, output=None):
        """Celestial (lon, lat, cos psi, sin psi) of each detector at each time
        (python/proj/coords.py:211-237)."""
        import so3g_gb300
        p = so3g_gb300.ProjEng_CAR_TQU_NonTiled((1, 1, 1., 1., 1., 1.))
        collapse = (fplane is None)
        if collapse:
            fplane = FocalPlane.boresight()
            if output is not None:
                output = output[None]
        output = p.coords(self.Q, fplane.quats, output)
        if collapse:
            output = output[0]
        return output


class FocalPlane:
    """Detector offset quaternions (``quats``, a G3VectorQuat) and (T, P)
    responses (``resps``, float32 [ndet, 2]) (python/proj/coords.py:239-434)."""

    def __init__(self, quats=None, resps=None, dets=None):
        if quats is None:
            quats = []
        self.quats = quat.G3VectorQuat(np.asarray(quats, dtype=np.float64).reshape(-1, 4)
                                       if not isinstance(quats, quat.G3VectorQuat) else quats)
        self.resps = np.ones((len(self.quats), 2), np.float32)
        if resps is not None:
            self.resps[:] = resps
        if np.any(~np.isfinite(np.asarray(self.quats))):
            raise ValueError("nan/inf values in detector quaternions")
        if np.any(~np.isfinite(self.resps)):
            raise ValueError("nan/inf values in detector responses")
        self._dets = list(dets) if dets is not None else []

    def coeffs(self):
        return np.array(self.quats, dtype=np.float64)

    @classmethod
    def boresight(cls):
        return cls(quats=[[1, 0, 0, 0]])

    @classmethod
    def from_xieta(cls, xi, eta, gamma=0, T=1, P=1, Q=1, U=0, hwp=False, dets=None):
        """Focal plane from (xi, eta) positions and polarisation angles gamma
        (python/proj/coords.py:305-381)."""
        gamma = gamma + np.arctan2(U, Q) / 2
        P = P * (Q ** 2 + U ** 2) ** 0.5
        if hwp:
            gamma = -gamma
        xi, eta, gamma, T, P, _ = np.broadcast_arrays(xi, eta, gamma, T, P, [0])
        quats = quat.rotation_xieta(xi, eta, gamma)
        resps = np.ones((len(quats), 2))
        resps[:, 0] = T
        resps[:, 1] = P
        return cls(quats, resps=resps, dets=dets)

    def __repr__(self):
        return "FocalPlane(quats=%s,resps=%s)" % (repr(self.coeffs()), repr(self.resps))

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
        for q, resp in zip(self.quats, self.resps):
            yield q, resp


class Assembly:
    """A boresight (``Q``) with rigidly attached detectors (``fplane``)."""

    def __init__(self, collapse=False):
        self.collapse = collapse

    @classmethod
    def attach(cls, sight_line, fplane):
        self = cls()
        if isinstance(sight_line, quat.G3VectorQuat):
            self.Q = sight_line
        else:
            self.Q = sight_line.Q
        self.fplane = fplane
        return self

    @classmethod
    def for_boresight(cls, sight_line):
        self = cls(collapse=True)
        self.Q = sight_line.Q
        self.fplane = FocalPlane.boresight()
        return self

    @property
    def dets(self):
        return self.fplane
