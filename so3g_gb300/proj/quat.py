"""Quaternion helpers of so3g.proj.quat (python/proj/quat.py:1-154) on a
numpy quaternion type.

so3g stores quaternions in spt3g's ``quat`` and ``G3VectorQuat`` with
component order (1, i, j, k).  Here ``quat`` is a single quaternion and
``G3VectorQuat`` an (n, 4) float64 ndarray subclass whose ``*`` is the
Hamilton product (broadcasting quat x vector, vector x quat and vector x
vector elementwise).  The product sums each component left to right.
"""
import numpy as np

DEG = np.pi / 180


def _qmul(p, q):
    p = np.asarray(p, dtype=np.float64)
    q = np.asarray(q, dtype=np.float64)
    a1, b1, c1, d1 = p[..., 0], p[..., 1], p[..., 2], p[..., 3]
    a2, b2, c2, d2 = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    return np.stack([
        a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2,
        a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2,
        a1 * c2 - b1 * d2 + c1 * a2 + d1 * b2,
        a1 * d2 + b1 * c2 - c1 * b2 + d1 * a2,
    ], axis=-1)


def _is_quat_like(x):
    return isinstance(x, (quat, G3VectorQuat))


class quat:
    """A single quaternion (a, b, c, d) = a + b i + c j + d k."""

    __slots__ = ("_v",)

    def __init__(self, a=0., b=0., c=0., d=0.):
        self._v = np.array([a, b, c, d], dtype=np.float64)

    a = property(lambda s: float(s._v[0]))
    b = property(lambda s: float(s._v[1]))
    c = property(lambda s: float(s._v[2]))
    d = property(lambda s: float(s._v[3]))

    def __array__(self, dtype=None, copy=None):
        return self._v.astype(dtype) if dtype is not None else self._v.copy()

    def __iter__(self):
        return iter(self._v.tolist())

    def __len__(self):
        return 4

    def __getitem__(self, i):
        return float(self._v[i])

    def __mul__(self, other):
        if isinstance(other, quat):
            return quat(*_qmul(self._v, other._v))
        if isinstance(other, G3VectorQuat):
            return G3VectorQuat(_qmul(self._v[None, :], np.asarray(other)))
        return quat(*(self._v * other))

    def __rmul__(self, other):
        return quat(*(self._v * other))

    def __truediv__(self, other):
        return quat(*(self._v / other))

    def __invert__(self):
        return quat(self._v[0], -self._v[1], -self._v[2], -self._v[3])

    def __neg__(self):
        return quat(*(-self._v))

    def __eq__(self, other):
        return isinstance(other, quat) and bool(np.all(self._v == other._v))

    def __abs__(self):
        return float(np.sqrt(np.sum(self._v ** 2)))

    def __repr__(self):
        return "quat(%r, %r, %r, %r)" % tuple(self._v.tolist())


class G3VectorQuat(np.ndarray):
    """A vector of quaternions: an (n, 4) float64 array."""

    def __new__(cls, data=()):
        if isinstance(data, quat):
            data = [np.asarray(data)]
        arr = np.array(data, dtype=np.float64)
        if arr.size == 0:
            arr = arr.reshape(0, 4)
        if arr.ndim == 1 and len(arr) and isinstance(data, (list, tuple)) and \
                all(isinstance(x, quat) for x in data):
            arr = np.array([np.asarray(x) for x in data])
        arr = arr.reshape(-1, 4)
        return arr.view(cls)

    def __getitem__(self, idx):
        r = np.ndarray.__getitem__(self, idx)
        if isinstance(idx, (int, np.integer)):
            return quat(*np.asarray(r))
        if isinstance(r, np.ndarray) and r.ndim == 2 and r.shape[-1] == 4:
            return r.view(G3VectorQuat)
        return np.asarray(r)

    def __setitem__(self, idx, value):
        self.view(np.ndarray)[idx] = np.asarray(value)

    def __mul__(self, other):
        if isinstance(other, quat):
            return G3VectorQuat(_qmul(np.asarray(self), np.asarray(other)[None, :]))
        if isinstance(other, G3VectorQuat):
            return G3VectorQuat(_qmul(np.asarray(self), np.asarray(other)))
        return np.multiply(np.asarray(self), other).view(G3VectorQuat)

    def __rmul__(self, other):
        if isinstance(other, quat):
            return G3VectorQuat(_qmul(np.asarray(other)[None, :], np.asarray(self)))
        return np.multiply(other, np.asarray(self)).view(G3VectorQuat)

    def __imul__(self, other):
        res = self * other
        self.view(np.ndarray)[...] = np.asarray(res)
        return self

    def __invert__(self):
        v = np.asarray(self).copy()
        v[:, 1:] *= -1
        return v.view(G3VectorQuat)

    def __iter__(self):
        for row in np.asarray(self):
            yield quat(*row)

    def append(self, q):
        raise TypeError("G3VectorQuat is fixed-size here; build a new one instead")


def euler(axis, angle):
    """Quaternion(s) of an Euler rotation about cartesian axis 0, 1 or 2:
    (cos(angle/2), .., sin(angle/2) at index axis+1, ..)
    (python/proj/quat.py:15-44)."""
    angle = np.asarray(angle)
    shape = np.broadcast(axis, angle).shape + (4,)
    c, s = np.cos(angle / 2), np.sin(angle / 2)
    q = np.zeros(shape)
    q[..., 0] = c
    q[..., axis + 1] = s
    if len(shape) == 1:
        return quat(*q)
    return G3VectorQuat(q)


def rotation_iso(theta, phi, psi=None):
    """Qz(phi) Qy(theta) Qz(psi) (python/proj/quat.py:47-57)."""
    output = euler(2, phi) * euler(1, theta)
    if psi is None:
        return output
    return output * euler(2, psi)


def rotation_lonlat(lon, lat, psi=0., azel=False):
    """Qz(lon) Qy(pi/2 - lat) Qz(psi) (python/proj/quat.py:60-73)."""
    if azel:
        return rotation_iso(np.pi / 2 - lat, -lon, psi)
    return rotation_iso(np.pi / 2 - lat, lon, psi)


def rotation_xieta(xi, eta, gamma=0):
    """Rotation taking the focal-plane centre to (xi, eta, gamma)
    (python/proj/quat.py:75-93)."""
    phi = np.arctan2(-xi, -eta)
    theta = np.arcsin(np.sqrt(np.asarray(xi) ** 2 + np.asarray(eta) ** 2))
    psi = gamma - phi
    return rotation_iso(theta, phi, psi)


def _components(q):
    if isinstance(q, quat):
        return q.a, q.b, q.c, q.d
    return tuple(np.transpose(np.asarray(q)))


def decompose_iso(q):
    """(theta, phi, psi) with q = Qz(phi) Qy(theta) Qz(psi)
    (python/proj/quat.py:95-124)."""
    a, b, c, d = _components(q)
    psi = np.arctan2(a * b + c * d, a * c - b * d)
    phi = np.arctan2(c * d - a * b, a * c + b * d)
    theta = 2 * np.arctan2((b ** 2 + c ** 2) ** .5, (a ** 2 + d ** 2) ** .5)
    return (theta, phi, psi)


def decompose_lonlat(q, azel=False):
    theta, phi, psi = decompose_iso(q)
    if azel:
        return (-phi, np.pi / 2 - theta, psi)
    return (phi, np.pi / 2 - theta, psi)


def decompose_xieta(q):
    a, b, c, d = _components(q)
    return (2 * (a * b - c * d), -2 * (a * c + b * d), np.arctan2(2 * a * d, a * a - d * d))
