"""Seeded synthetic observations for tests and benchmarks.

A constant-elevation scan (triangle-wave azimuth, python/proj/util.py:4-25)
in the horizon model of CelestialSightLine.for_horizon
(python/proj/coords.py:190-209), a hexagonal focal plane built with
rotation_xieta (python/proj/quat.py:75-93), random polarisation angles,
unit (T, P) responses, and a map geometry centred on the scan.  Draw order
from ``numpy.random.default_rng(seed)`` is fixed: detector layout, then
polarisation angles, then the signal.
"""
import numpy as np

from .proj import quat
from .proj.util import ces
from .proj.geometry import SimpleWCS
from .proj.wcs import Projectionist

DEG = np.pi / 180
ARCMIN = DEG / 60


def hex_layout(n_det, radius):
    """First n_det points of a hexagonal lattice ordered by radius, scaled
    so the outermost point sits at `radius` (radians).  Returns (xi, eta)."""
    k = int(np.ceil(np.sqrt(n_det))) + 2
    ii, jj = np.meshgrid(np.arange(-k, k + 1), np.arange(-k, k + 1))
    x = (ii + 0.5 * jj).ravel()
    y = (jj * np.sqrt(3) / 2).ravel()
    r = np.hypot(x, y)
    order = np.lexsort((np.arctan2(y, x), np.round(r, 9)))[:n_det]
    x, y, r = x[order], y[order], r[order]
    scale = radius / max(r.max(), 1e-12) if n_det > 1 else 0.
    return x * scale, y * scale


def scan(n_time, rate=200., el=50., az0=180., throw=10., v_az=1., drift_deg_per_hour=0.,
         t0=1700000000.):
    """Boresight quaternions (n_time, 4) of a CES; angles in degrees."""
    t = t0 + np.arange(n_time) / rate
    az, el_v = ces(el, az0, throw, v_az, t)
    if drift_deg_per_hour:
        az = az + drift_deg_per_hour * (t - t0) / 3600.
    Q = quat.euler(2, -az * DEG) * quat.euler(1, np.pi / 2 - el_v * DEG) * quat.euler(2, 0.)
    return np.asarray(Q), t


def focal_plane(rng, n_det, radius_deg):
    xi, eta = hex_layout(n_det, radius_deg * DEG)
    gamma = rng.uniform(0, np.pi, n_det)
    dets = np.asarray(quat.rotation_xieta(xi, eta, gamma)).reshape(-1, 4)
    resp = np.ones((n_det, 2), dtype=np.float32)
    return dets, resp, gamma


def car_projectionist(shape, res, el=50., az0=180., proj='CAR', tile_shape=None,
                      interpol=None):
    """Projectionist for a map centred on the scan centre (lon = -az0, lat
    = el), so the scan sits near the native equator."""
    ny, nx = shape
    r = np.degrees(res)
    wcs = SimpleWCS(proj, (-az0, el), (-r, r), (nx / 2. + 0.5, ny / 2. + 0.5))
    if tile_shape is not None:
        return Projectionist.for_tiled((ny, nx), wcs, tile_shape, interpol=interpol)
    return Projectionist.for_geom((ny, nx), wcs, interpol=interpol)


def workload(n_det, n_time, seed=0, radius_deg=1.0, rate=200., el=50., az0=180., throw=10.,
             v_az=1., signal=True):
    """(q_bore, dets, resp, gamma, signal) of a seeded CES observation.
    q_bore is in the celestial (here: horizon) frame; rotate it with a
    Projectionist's q_celestial_to_native before projecting."""
    rng = np.random.default_rng(seed)
    dets, resp, gamma = focal_plane(rng, n_det, radius_deg)
    Q, t = scan(n_time, rate, el, az0, throw, v_az)
    sig = rng.standard_normal((n_det, n_time), dtype=np.float32) if signal else None
    return Q, dets, resp, gamma, sig


def native(proj, Q):
    """q_native = q_celestial_to_native * Q as a plain (n, 4) array."""
    return np.ascontiguousarray(np.asarray(proj.q_celestial_to_native *
                                           quat.G3VectorQuat(Q)), dtype=np.float64)


# The benchmark workloads: focal plane radius (deg), scan (el, az throw and
# speed in deg and deg/s, azimuth drift in deg/hour) and map of each.
#   car  -- CAR TQU map of `shape` pixels at `res_arcmin`, centred on the scan
#   hp   -- HEALPix TQU, RING untiled or NEST tiled (nside_tile)
#   zea  -- ZEA bilinear TQU map, as car
WORKLOADS = {
    "cfg1": dict(kind="car", n_det=64, n_time=100_000, radius=1.0, shape=(600, 600),
                 res_arcmin=1.0, el=50., throw=10., v_az=1., drift=0.),
    "cfg2": dict(kind="car", n_det=1000, n_time=1_000_000, radius=1.5, shape=(2000, 2000),
                 res_arcmin=1.0, el=50., throw=10., v_az=1., drift=0.),
    "cfg3": dict(kind="hp", n_det=2000, n_time=2_000_000, radius=1.5, nside=1024,
                 nside_tile=16, el=45., throw=30., v_az=2., drift=15.),
    "cfg5": dict(kind="zea", n_det=4000, n_time=2_000_000, radius=1.5, shape=(3000, 3000),
                 res_arcmin=0.5, el=50., throw=10., v_az=1., drift=0.),
}


def projection_inputs(c, seed=0, dets=None, tiled=False, tile_shape=(100, 100)):
    """(projectionist, q_native (n_time, 4), dets (n_det, 4), resp (n_det, 2))
    of a workload dict `c` (WORKLOADS entries, possibly with n_det/n_time
    changed).  `dets` selects detectors of the full focal plane (e.g. every
    20th, so a slice keeps the focal plane's footprint).  tiled: the NEST
    tiled HEALPix map (nside_tile), or a flat map cut into tile_shape tiles
    with every tile present."""
    from .proj.wcs import ProjectionistHealpix
    rng = np.random.default_rng(seed)
    d, resp, _ = focal_plane(rng, c["n_det"], c["radius"])
    if dets is not None:
        d, resp = d[dets], resp[dets]
    el = c.get("el", 50.)
    Q, _ = scan(c["n_time"], rate=200., el=el, az0=180., throw=c.get("throw", 10.),
                v_az=c.get("v_az", 1.), drift_deg_per_hour=c.get("drift", 0.))
    kind = c.get("kind", "car")
    if kind == "hp":
        if tiled:
            nt = 12 * c["nside_tile"] ** 2
            p = ProjectionistHealpix.for_healpix(c["nside"], nside_tile=c["nside_tile"],
                                                 active_tiles=list(range(nt)), ordering="NEST")
        else:
            p = ProjectionistHealpix.for_healpix(c["nside"], ordering="RING")
    elif kind == "zea":
        p = car_projectionist(c["shape"], c["res_arcmin"] * ARCMIN, el=el, az0=180.,
                              proj="ZEA", interpol="bilinear")
    else:
        p = car_projectionist(c["shape"], c.get("res_arcmin", 1.) * ARCMIN, el=el, az0=180.,
                              proj=c.get("proj", "CAR"),
                              tile_shape=tile_shape if tiled else None)
    return p, native(p, Q), np.ascontiguousarray(d), np.ascontiguousarray(resp)
