"""Boresight generation on the device (CelestialSightLine.for_horizon and
naive_az_el with CUDA tensors in, python/proj/coords.py:99-125, 190-209) and
the device form of Projectionist._cache_q_fp_to_native
(python/proj/wcs.py:140-148), against the numpy evaluation of the same
expressions.  The kernels repeat numpy's operations in order; only cos/sin
may differ in the last bit, so quaternions agree to a few ulp and pixel
indices exactly."""
import numpy as np
import pytest

from so3g_gb300 import synth
from so3g_gb300.proj import coords, quat

pytestmark = pytest.mark.gpu

DEG = np.pi / 180


def scan_inputs(n=200_000, seed=3):
    rng = np.random.default_rng(seed)
    t = 1.7e9 + np.arange(n) / 200.
    az, el = synth.ces(50., 180., 10., 1., t)
    az = az * DEG + rng.normal(0, 1e-4, n)
    el = el * DEG + rng.normal(0, 1e-4, n)
    roll = rng.uniform(-0.3, 0.3, n)
    return t, az, el, roll


def dev(x):
    import torch
    return torch.as_tensor(x, dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("roll_kind", ["none", "scalar", "vector"])
def test_for_horizon_matches_numpy(gpulib, roll_kind):
    t, az, el, roll = scan_inputs()
    r = {"none": None, "scalar": 0.123, "vector": roll}[roll_kind]
    host = np.asarray(coords.CelestialSightLine.for_horizon(t, az, el, r).Q)
    rd = dev(r) if roll_kind == "vector" else r
    got = coords.CelestialSightLine.for_horizon(dev(t), dev(az), dev(el), rd).Q
    got = got.cpu().numpy()
    assert got.shape == host.shape == (len(t), 4)
    assert np.abs(got - host).max() <= 1e-15
    # Most samples agree to the last bit.
    assert np.mean(np.all(got == host, axis=1)) > 0.5


def test_naive_az_el_matches_numpy(gpulib):
    t, az, el, roll = scan_inputs()
    site = coords.SITES["so"]
    host = np.asarray(coords.CelestialSightLine.naive_az_el(t, az, el, roll=0.2, site=site).Q)
    got = coords.CelestialSightLine.naive_az_el(dev(t), dev(az), dev(el), roll=0.2,
                                                site=site).Q.cpu().numpy()
    # lst is ~6e4 rad: its cos/sin carry the argument's own rounding
    # (ulp(6e4) ~ 7e-12) identically on both sides; what may differ is the
    # last bit of the results.
    assert np.abs(got - host).max() <= 4e-15


def test_scalar_elevation_broadcasts(gpulib):
    t, az, el, _ = scan_inputs(5000)
    host = np.asarray(coords.CelestialSightLine.for_horizon(t, az, 0.8).Q)
    got = coords.CelestialSightLine.for_horizon(dev(t), dev(az), 0.8).Q.cpu().numpy()
    assert np.abs(got - host).max() <= 1e-15


def test_left_multiply_bit_exact(gpulib):
    from so3g_gb300 import sightline
    t, az, el, roll = scan_inputs(50_000)
    Q = np.asarray(coords.CelestialSightLine.for_horizon(t, az, el, roll).Q)
    q = quat.euler(1, 0.7) * quat.euler(2, -1.2)
    want = np.asarray(q * quat.G3VectorQuat(Q))
    got = sightline.left_multiply(q, dev(Q)).cpu().numpy()
    assert np.array_equal(got.view(np.int64), want.view(np.int64))


def test_projectionist_with_device_boresight(gpulib):
    """A device sight line through Projectionist.to_map / get_pixels: the
    same pixels and map as the host sight line."""
    import torch
    t, az, el, roll = scan_inputs(100_000)
    p = synth.car_projectionist((600, 600), 1. / 60 * DEG)
    rng = np.random.default_rng(0)
    dq, resp, _ = synth.focal_plane(rng, 16, 1.0)
    fp = coords.FocalPlane(quats=dq, resps=resp)
    sig = rng.standard_normal((16, len(t)), dtype=np.float32)
    a_host = coords.Assembly.attach(coords.CelestialSightLine.for_horizon(t, az, el, roll), fp)
    a_dev = coords.Assembly.attach(
        coords.CelestialSightLine.for_horizon(dev(t), dev(az), dev(el), dev(roll)), fp)
    pix_h = np.array(p.get_pixels(a_host))
    pix_d = np.array([np.asarray(x.cpu() if hasattr(x, "cpu") else x)
                      for x in p.get_pixels(a_dev)])
    assert np.array_equal(pix_h, pix_d)
    m_h = np.asarray(p.to_map(sig, a_host, comps="TQU"))
    m_d = p.to_map(torch.as_tensor(sig, device="cuda"), a_dev, comps="TQU")
    m_d = m_d.cpu().numpy() if hasattr(m_d, "cpu") else np.asarray(m_d)
    scale = np.abs(m_h).max()
    assert scale > 0
    assert np.abs(m_d - m_h).max() <= 1e-12 * scale


def test_bad_inputs_raise(gpulib):
    t, az, el, _ = scan_inputs(100)
    with pytest.raises(ValueError):
        coords.CelestialSightLine.for_horizon(dev(t), dev(az), dev(el[:50]))
    with pytest.raises(ValueError):
        coords.CelestialSightLine.for_horizon(dev(t), dev(az).reshape(10, 10), dev(el))
