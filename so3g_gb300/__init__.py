"""so3g_gb300 -- so3g's ProjectionEngine hot path, native on NVIDIA GB300.

The package provides the ``ProjEng_*`` classes of so3g (quaternion
pointing, CAR/CEA/ARC/SIN/TAN/ZEA/Flat/Quat and HEALPix pixelizations,
NonTiled and Tiled, nearest and bilinear, SpinT/SpinQU/SpinTQU; to_map,
to_weight_map, from_map and the pointing queries), plus ``RangesInt32``,
``useful_info()`` and ``version()``, under the names so3g uses, and
``so3g_gb300.proj`` mirrors ``so3g.proj`` (Projectionist,
ProjectionistHealpix, quaternion helpers, FocalPlane, Assembly, ...).

All projection work runs in the CUDA library built from so3g_gb300/csrc
(see so3g_gb300.build); the Python layer validates arguments, moves data
and maps errors to so3g's exception classes.

``install_as_so3g()`` registers this package under the module name
``so3g`` so that code written against so3g imports it unchanged.
"""
import os
import sys

import numpy as np

from .ranges import RangesInt32, RangesMatrix  # noqa: F401
from .projeng import ENGINES, ProjEngBase, ProjEngPrecompBase  # noqa: F401

globals().update(ENGINES)

__version__ = "0.1.0"


def version():
    return __version__


def set_chunked_min_samples(n):
    """Sets the smallest call (detectors x samples, whole detectors) that
    takes the chunked mixed-pointing kernels; returns the previous value
    (default 3e7: smaller calls take the per-sample float32 tier, whose
    fixed cost per call is lower).  Process-wide."""
    from . import _abi
    return int(_abi.lib().so3g_set_chunked_min_samples(int(n)))


def useful_info():
    """so3g's useful_info() (src/main.cxx:26-39).  omp_num_threads is the
    host thread count used by the thread-assignment helpers."""
    n = os.environ.get("OMP_NUM_THREADS")
    try:
        n = int(n) if n else (os.cpu_count() or 1)
    except ValueError:
        n = os.cpu_count() or 1
    return {"omp_num_threads": n, "version": __version__, "backend": "cuda-sm_103a"}


def test_trig(table_size=1 << 14, verbose=0):
    """Worst absolute error of the asin/atan2 interpolation tables against
    the math library over so3g's test grid (src/so_linterp.cxx:8-36).  A
    diagnostic: it reads the library's host tables and interpolates them
    with numpy."""
    from . import _abi
    if table_size != _abi.LUT_N:
        raise ValueError("the library's tables have %d entries" % _abi.LUT_N)
    a = np.empty(_abi.LUT_N)
    b = np.empty(_abi.LUT_N)
    _abi.check(_abi.lib().so3g_get_trig_tables(a.ctypes.data, b.ctypes.data, _abi.LUT_N),
               "get_trig_tables")
    n = _abi.LUT_N
    dx = 1. / (n - 1)

    def raw(v, x):
        d = x / dx
        if x < 0:
            return v[0]
        if d >= n - 1:
            return v[n - 1]
        i = int(d)
        d -= i
        return v[i] * (1 - d) + v[i + 1] * d

    def asin_t(x):
        return -raw(a, -x) if x < 0 else raw(a, x)

    def atan2_t(y, x):
        if y < 0:
            return -atan2_t(-y, x)
        if x < 0:
            return np.pi - atan2_t(y, -x)
        if y == 0:
            return b[0]
        if x < y:
            return np.pi / 2 - raw(b, x / y)
        return raw(b, y / x)

    worst = 0.
    x = -1.
    while x < 1.:
        worst = max(worst, abs(asin_t(x) - np.arcsin(x)))
        x += .01
    gx = -3.
    while gx < 3.1:
        gy = -1.
        while gy < 1.:
            worst = max(worst, abs(atan2_t(gy, gx) - np.arctan2(gy, gx)))
            gy += .01
        gx += 0.5
    return float(worst)


def install_as_so3g():
    """Make ``import so3g`` / ``import so3g.proj`` resolve to this package."""
    from . import proj
    sys.modules.setdefault("so3g", sys.modules[__name__])
    sys.modules.setdefault("so3g.proj", proj)
    return sys.modules["so3g"]
