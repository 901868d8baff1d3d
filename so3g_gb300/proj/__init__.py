"""so3g_gb300.proj -- the so3g.proj API (python/proj/__init__.py) over the
GB300 ProjectionEngine."""
import numpy as np

from . import quat  # noqa: F401
from . import util  # noqa: F401
from . import mapthreads  # noqa: F401
from .wcs import Projectionist, ProjectionistHealpix, Ranges, RangesMatrix  # noqa: F401
from .coords import CelestialSightLine, EarthlySite, Assembly, FocalPlane, SITES  # noqa: F401
from .geometry import SimpleWCS, geometry  # noqa: F401

DEG = np.pi / 180.
