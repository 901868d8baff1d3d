"""A minimal celestial WCS for Projectionist.for_geom.

Projectionist reads a WCS through the attributes of astropy's ``wcs.wcs``
(crval, cdelt, crpix, ctype, lng, lat, phi0, theta0, lonpole) and
``.celestial``.  ``SimpleWCS`` carries exactly those, and ``geometry()``
builds a (shape, wcs) pair for a map centred on a sky position in the
conventions pixell uses for CAR (cylindrical, reference point at the map
centre) and the zenithal projections (TAN, ZEA, ARC, SIN, reference point
at the native pole).  astropy and pixell objects work unchanged where they
are installed.
"""
import numpy as np

CYLINDRICAL = ('CAR', 'CEA')
ZENITHAL = ('TAN', 'ZEA', 'ARC', 'SIN')


class _WcsParams:
    def __init__(self, ctype, crval, cdelt, crpix, phi0, theta0, lonpole):
        self.ctype = list(ctype)
        self.crval = np.array(crval, dtype=float)
        self.cdelt = np.array(cdelt, dtype=float)
        self.crpix = np.array(crpix, dtype=float)
        self.phi0 = float(phi0)
        self.theta0 = float(theta0)
        self.lonpole = float(lonpole)
        self.lng = 0
        self.lat = 1


class SimpleWCS:
    """Celestial WCS with axes (lon, lat) = (x, y); angles in degrees."""

    def __init__(self, proj, crval, cdelt, crpix, lonpole=None):
        proj = proj.upper()
        if proj in CYLINDRICAL:
            phi0, theta0 = 0., 0.
            if lonpole is None:
                lonpole = 180. if crval[1] >= 0 else 0.
        elif proj in ZENITHAL:
            phi0, theta0 = 0., 90.
            if lonpole is None:
                lonpole = 180.
        else:
            raise ValueError("unsupported projection %s" % proj)
        self.wcs = _WcsParams(['RA---' + proj, 'DEC--' + proj], crval, cdelt, crpix,
                              phi0, theta0, lonpole)

    @property
    def celestial(self):
        return self

    def __repr__(self):
        w = self.wcs
        return "SimpleWCS(%s, crval=%s, cdelt=%s, crpix=%s)" % (
            w.ctype[0][-3:], list(w.crval), list(w.cdelt), list(w.crpix))


def geometry(pos, res, shape, proj='CAR'):
    """(shape, wcs) of a map of `shape` (ny, nx) pixels of `res` radians
    centred on pos = (dec, ra) radians.  RA increases to the left (cdelt_x
    < 0), as on the sky."""
    dec0, ra0 = (np.degrees(p) for p in pos)
    r = np.degrees(res)
    ny, nx = shape[-2:]
    crpix = (nx / 2. + 0.5, ny / 2. + 0.5)
    w = SimpleWCS(proj, (ra0, dec0), (-r, r), crpix)
    return tuple(shape), w
