"""Scan helpers of so3g.proj.util (python/proj/util.py:4-25)."""
import numpy as np


def ces(el, az0, throw, v_scan, t):
    """Constant-elevation scan: az is a triangle wave of half-amplitude
    ``throw`` about ``az0`` at speed ``v_scan``; returns (az, el) vectors
    the length of t (any consistent angle and time units)."""
    t = np.asarray(t, dtype=np.float64)
    phase = (t - t[0]) * v_scan % (4 * throw)
    az = phase.copy()
    back = phase > 2 * throw
    az[back] = 4 * throw - phase[back]
    return az - throw + az0, el + az * 0
