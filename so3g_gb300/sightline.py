"""Boresight generation on the device: CelestialSightLine.for_horizon and
naive_az_el (python/proj/coords.py:99-125, 190-209) for az/el/time given as
CUDA tensors, and the quat x vector product of
Projectionist._cache_q_fp_to_native (python/proj/wcs.py:140-148) for a
boresight held on the device.  Both run the library's kernels
(so3g_boresight, so3g_quat_left_multiply); the constants are formed here
exactly as the numpy code path forms them, so the two paths differ only
where the device's cos/sin differ from the host's in the last bit.
"""
import numpy as np
import torch

from . import _abi
from .projeng import _stream


def is_device(*xs):
    """True if any argument is a CUDA tensor."""
    return any(isinstance(x, torch.Tensor) and x.is_cuda for x in xs)


def _device_of(*xs):
    for x in xs:
        if isinstance(x, torch.Tensor) and x.is_cuda:
            return x.device
    raise ValueError("no CUDA tensor among the arguments")


def _vector(x, n, dev, name):
    """x as a contiguous float64 CUDA vector of length n (scalars broadcast)."""
    if isinstance(x, torch.Tensor):
        x = x.to(device=dev, dtype=torch.float64)
    else:
        x = torch.as_tensor(np.asarray(x, dtype=np.float64), device=dev)
    if x.dim() == 0:
        x = x.expand(n)
    if x.dim() != 1 or x.shape[0] != n:
        raise ValueError("%s: expected a scalar or a vector of %d samples, got shape %s"
                         % (name, n, tuple(x.shape)))
    return x.contiguous()


def _length(*xs):
    n = None
    for x in xs:
        if x is None:
            continue
        shape = tuple(x.shape) if isinstance(x, torch.Tensor) else np.shape(x)
        if len(shape) == 0:
            continue
        if len(shape) != 1:
            raise ValueError("sight-line inputs must be scalars or vectors")
        if n is not None and shape[0] != n:
            raise ValueError("sight-line vectors differ in length (%d, %d)" % (n, shape[0]))
        n = shape[0]
    if n is None:
        raise ValueError("at least one of t, az, el must be a vector")
    return n


def _quat4(q):
    """A quaternion as the 4 float64 of a ctypes struct field."""
    return (_abi.c_double * 4)(*np.asarray(q, dtype=np.float64).reshape(4).tolist())


def _is_scalar(x):
    if isinstance(x, torch.Tensor):
        return x.dim() == 0
    return np.ndim(x) == 0


def boresight(kind, t, az, el, roll=None, site=None, q_left=None):
    """Boresight quaternions (n, 4) float64 on the device.

    kind: "horizon" (for_horizon) or "naive" (naive_az_el, which needs t and
    an EarthlySite `site`).  roll: scalar, vector or None (0).  q_left: an
    optional constant quaternion multiplied on the left."""
    from .proj import quat
    from .proj.coords import DEG, ERA_EPOCH, ERA_POLY
    dev = _device_of(t, az, el, roll)
    n = _length(t if kind == "naive" else None, az, el, roll)
    sl = _abi.SightLine()
    if kind == "horizon":
        sl.kind = _abi.SIGHT_HORIZON
    elif kind == "naive":
        sl.kind = _abi.SIGHT_NAIVE_AZEL
        sl.site_lon_rad = site.lon * DEG
        sl.era_epoch = float(ERA_EPOCH)
        sl.era_poly = (_abi.c_double * 2)(*ERA_POLY.tolist())
        sl.q_site_lat = _quat4(quat.euler(1, np.pi / 2 - site.lat * DEG))
        sl.q_pi = _quat4(quat.euler(2, np.pi))
    else:
        raise ValueError("unknown sight-line kind %r" % (kind,))
    with torch.cuda.device(dev):
        t_d = _vector(t, n, dev, "t") if kind == "naive" else None
        az_d = _vector(az, n, dev, "az")
        el_d = _vector(el, n, dev, "el")
        roll_d = None
        if roll is None:
            sl.roll = 0.
        elif _is_scalar(roll):
            sl.roll = float(roll)
        else:
            roll_d = _vector(roll, n, dev, "roll")
        if q_left is not None:
            sl.has_left = 1
            sl.q_left = _quat4(q_left)
        out = torch.empty((n, 4), dtype=torch.float64, device=dev)
        _abi.check(_abi.lib().so3g_boresight(
            sl, None if t_d is None else t_d.data_ptr(), az_d.data_ptr(), el_d.data_ptr(),
            None if roll_d is None else roll_d.data_ptr(), n, out.data_ptr(), _stream()),
            "boresight")
    return out


def left_multiply(q_left, Q):
    """q_left * Q[i] for a device boresight Q (n, 4) float64."""
    dev = Q.device
    Q = Q.to(torch.float64).contiguous()
    if Q.dim() != 2 or Q.shape[1] != 4:
        raise ValueError("expected an (n, 4) quaternion array, got shape %s" % (tuple(Q.shape),))
    with torch.cuda.device(dev):
        out = torch.empty_like(Q)
        left = np.ascontiguousarray(np.asarray(q_left, dtype=np.float64).reshape(4))
        _abi.check(_abi.lib().so3g_quat_left_multiply(
            left.ctypes.data, Q.data_ptr(), Q.shape[0], out.data_ptr(), _stream()),
            "quat_left_multiply")
    return out
