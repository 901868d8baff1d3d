"""Generates the golden vectors in tests/golden/ from the so3g reference.

The two pieces of so3g's ProjectionEngine that compile on their own --
include/so_linterp.h (asin/atan2 interpolation tables) and
src/healpix_bare.c (HEALPix ang2ring/ang2nest) -- are built from the
reference checkout by oracle/build.py:build_ref() into oracle/_ref/ and
evaluated here on seeded inputs.  The outputs pin the oracle's restatement
of those pieces (tests/test_oracle_golden.py).  Run from the repository
root where the reference checkout is present:

    python tests/golden/make_golden.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import build  # noqa: E402


def load_ref():
    path = build.build_ref()
    if path is None:
        raise SystemExit("reference checkout not found")
    L = ctypes.CDLL(path)
    d, ll, v = ctypes.c_double, ctypes.c_longlong, ctypes.c_void_p
    L.ref_asin.restype = d
    L.ref_asin.argtypes = [d]
    L.ref_atan2.restype = d
    L.ref_atan2.argtypes = [d, d]
    L.ref_tables.argtypes = [v, v, ctypes.c_int]
    L.ref_ang2ring.restype = ll
    L.ref_ang2ring.argtypes = [ll, d, d]
    L.ref_ang2nest.restype = ll
    L.ref_ang2nest.argtypes = [ll, d, d]
    L.ref_nest2ring.restype = ll
    L.ref_nest2ring.argtypes = [ll, ll]
    L.ref_trig_worst.restype = d
    L.ref_trig_worst.argtypes = [ctypes.c_int]
    return L


def trig_inputs(rng):
    xs = np.concatenate([
        rng.uniform(-1.05, 1.05, 2000),
        np.linspace(-1, 1, 501),
        np.arange(0, 16384) / 16383.,           # every knot of the table
        [0., 1., -1., 1. + 1e-12, -1. - 1e-12, 1e-300, -1e-300, 0.5, -0.5],
    ])
    ys = np.concatenate([rng.normal(size=2000), [0., 0., 1., -1., 1., -1., 1e-8, 3., 2.]])
    xx = np.concatenate([rng.normal(size=2000), [1., -1., 0., 0., 1., -1., 1., 3., -2.]])
    # Points on the octant boundaries |y| = |x|.
    b = rng.uniform(0.1, 2, 200)
    ys = np.concatenate([ys, b, -b, b, -b])
    xx = np.concatenate([xx, b, b, -b, -b])
    return xs, ys, xx


def healpix_inputs(rng):
    n = 5000
    z = rng.uniform(-1, 1, n)
    theta = np.arccos(z)
    phi = rng.uniform(-2 * np.pi, 2 * np.pi, n)
    # Polar caps, the cap/equator boundary |z| = 2/3 and face seams.
    extra_t = np.concatenate([
        [0., np.pi, np.pi / 2, np.arccos(2. / 3), np.arccos(-2. / 3), 1e-9, np.pi - 1e-9],
        np.arccos(np.linspace(-1, 1, 101)),
    ])
    extra_p = np.concatenate([
        [0., 0., 0., 0., 0., 0., 0.],
        np.linspace(-np.pi, np.pi, 101),
    ])
    # phi = -2 pi itself is left out: healpix_bare's wrap of x = -1 leaves
    # x = -1 and indexes its face tables out of range there.
    seams_p = np.arange(-7, 9) * np.pi / 4
    seams_t = np.full(len(seams_p), 1.1)
    theta = np.concatenate([theta, extra_t, seams_t])
    phi = np.concatenate([phi, extra_p, seams_p])
    return theta, phi


def main():
    L = load_ref()
    rng = np.random.default_rng(20240601)
    xs, ys, xx = trig_inputs(rng)
    asin_out = np.array([L.ref_asin(x) for x in xs])
    atan2_out = np.array([L.ref_atan2(y, x) for y, x in zip(ys, xx)])
    ta = np.empty(1 << 14)
    tb = np.empty(1 << 14)
    assert L.ref_tables(ta.ctypes.data, tb.ctypes.data, 1 << 14) == 0
    np.savez_compressed(os.path.join(HERE, "trig_lut.npz"), asin_x=xs, asin_out=asin_out,
                        atan2_y=ys, atan2_x=xx, atan2_out=atan2_out, table_asin=ta,
                        table_atan2=tb, trig_worst=np.array(L.ref_trig_worst(1 << 14)))

    theta, phi = healpix_inputs(rng)
    nsides = np.array([1, 2, 16, 128, 1024, 4096], dtype=np.int64)
    ring = np.empty((len(nsides), len(theta)), dtype=np.int32)
    nest = np.empty_like(ring)
    for k, ns in enumerate(nsides):
        ring[k] = [L.ref_ang2ring(int(ns), t, p) for t, p in zip(theta, phi)]
        nest[k] = [L.ref_ang2nest(int(ns), t, p) for t, p in zip(theta, phi)]
    np.savez_compressed(os.path.join(HERE, "healpix_ang2pix.npz"), theta=theta, phi=phi,
                        nsides=nsides, ring=ring, nest=nest)
    print("wrote trig_lut.npz and healpix_ang2pix.npz")


if __name__ == "__main__":
    main()
