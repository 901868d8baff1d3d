"""Known-answer tests of the reference, ported onto the CPU oracle.

The reference's tests need pixell, qpoint and ephem, which are not
available; their assertions are restated here on the same kind of inputs
(built with this package's quaternion helpers) and run against the oracle,
which pins the oracle's restatement of the pointing, the pixelizors and the
spin factors to the reference's conventions."""
import numpy as np
import pytest

import so3g_gb300
from so3g_gb300.proj import quat, FocalPlane, SimpleWCS, Projectionist

DEG = np.pi / 180


def _polar_crossings(amp=10., b=0., det_gamma=0., angs=None):
    """Trajectories through (or near, at impact parameter b) the native
    pole (test/test_proj_zen.py:40-62)."""
    if angs is None:
        angs = np.arange(0, 180., 10.)
    xi0 = np.linspace(-amp, amp, 101) * DEG
    eta0 = 0 * xi0 + b * DEG
    xi, eta, gam = [], [], []
    for ang in angs:
        c, s = np.cos(ang * DEG), np.sin(ang * DEG)
        xi.append(xi0 * c - eta0 * s)
        eta.append(eta0 * c + xi0 * s)
        gam.append(xi0 * 0)
    xi, eta, gam = [np.hstack(x) for x in [xi, eta, gam]]
    Q = quat.rotation_xieta(xi, eta, gam)
    fp = FocalPlane.from_xieta([0.], [0.], [det_gamma * DEG])
    return Q, fp


@pytest.mark.parametrize("pix", ["arc", "sin", "tan", "zea"])
def test_zenithal_polarization_purity(orc, pix):
    """test/test_proj_zen.py:107-133: at 1 arcsec pixels near the pole,
    from_map of Q = cos(2*34 deg), U = sin(2*34 deg) gives
    cos(2 (34 deg - gamma_det)) to 1e-6."""
    res = 1 / 3600
    w = SimpleWCS(pix.upper(), (0., 90.), (-res, res), (250.5, 250.5))
    p = Projectionist.for_geom((500, 500), w)
    eng = p.get_ProjEng("TQU")
    pz = eng._pz()
    ang = 34 * DEG
    mm = np.zeros((3, 500, 500))
    mm[1] = np.cos(2 * ang)
    mm[2] = np.sin(2 * ang)
    for det_gamma in [0., 37.]:
        for b_impact in [0., .001, .010]:
            Q, fp = _polar_crossings(amp=.05, b=b_impact, det_gamma=det_gamma)
            q = np.asarray(p.q_celestial_to_native * Q)
            sig = np.zeros((1, len(q)), np.float32)
            orc.from_map(pz, q, fp.coeffs(), fp.resps, mm.ravel().copy(), sig)
            expected = np.cos(2 * (ang - det_gamma * DEG))
            np.testing.assert_allclose(sig, expected, rtol=0., atol=1e-6)


def test_focalplane_coords(orc):
    """test/test_proj_astro.py:196-230: CAR coords() of each detector
    equal decompose_lonlat(r * q_det) within 1 arcsec, gamma within
    0.01 deg."""
    xi = np.array([1., 0., 0.]) * DEG
    eta = np.array([0., 0., 1.]) * DEG
    gamma = np.array([45, 0, -45]) * DEG
    fp = FocalPlane.from_xieta(xi, eta, gamma)
    r = quat.rotation_lonlat(35 * DEG, 80 * DEG, 15 * DEG)
    Q = np.asarray(quat.G3VectorQuat([r]))
    pz = so3g_gb300.ProjEng_CAR_TQU_NonTiled((1, 1, 1., 1., 1., 1.))._pz()
    coords = orc.coords(pz, Q, fp.coeffs())
    for i, (roffset, resp) in enumerate(fp.items()):
        lon0, lat0, gamma0 = quat.decompose_lonlat(r * roffset)
        lon1, lat1, cosg, sing = coords[i][0]
        gamma1 = np.arctan2(sing, cosg)
        dlon = (lon1 - lon0 + np.pi) % (2 * np.pi) - np.pi
        assert abs(dlon * np.cos(lat0)) < 1. / 3600 * DEG
        assert abs(lat1 - lat0) < 1. / 3600 * DEG
        dg = (gamma1 - gamma0 + np.pi) % (2 * np.pi) - np.pi
        assert abs(dg) < 0.01 * DEG


def test_zero_det_weights_give_empty_map(orc):
    """test/test_proj_eng.py:71-74."""
    from so3g_gb300 import synth
    Q, dets, resp, gamma, sig = synth.workload(3, 2000, seed=2, rate=20., throw=2.)
    p = synth.car_projectionist((100, 150), 3 * DEG / 60)
    q = synth.native(p, Q)
    pz = p.get_ProjEng("TQU")._pz()
    m = np.zeros(3 * 100 * 150)
    orc.to_map(pz, q, dets, resp, sig, np.zeros(3, np.float32), m)
    assert np.all(m == 0)
    orc.to_map(pz, q, dets, resp, sig, None, m)
    assert np.any(m != 0)


def test_pixel_range_coverage(orc):
    """Every on-map sample is in exactly one stripe domain
    (test/test_proj_eng.py:103-151, 'simple' method)."""
    from so3g_gb300 import synth
    Q, dets, resp, gamma, sig = synth.workload(3, 2000, seed=2, rate=20., throw=2.)
    p = synth.car_projectionist((60, 80), 3 * DEG / 60)
    q = synth.native(p, Q)
    eng = p.get_ProjEng("T")
    pz = eng._pz()
    lab = orc.labels(pz, q, dets, 0, 3)
    pix = orc.pixels(pz, q, dets, 2)
    assert np.array_equal(lab >= 0, pix[..., 0] >= 0)
    assert lab.max() < 3
