"""ctypes view of the C ABI declared in include/so3g_gb300.h.

The structs here mirror the header field for field; ``lib()`` loads the
in-tree libso3g_gb300.so (built by so3g_gb300/build.py) and declares the
argument types of every entry point.  A missing library is an error: there
is no other implementation behind these calls.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libso3g_gb300.so")

# enum so3g_coord_sys
COORD = {"Flat": 0, "Quat": 1, "CAR": 2, "CEA": 3, "ARC": 4, "SIN": 5, "TAN": 6, "ZEA": 7}
PIX_FLAT, PIX_HEALPIX = 0, 1
INTERP_NEAREST, INTERP_BILINEAR = 0, 1
ACCUM_ATOMIC, ACCUM_WARP_RUNS = 0, 1
DEVERR_NONE, DEVERR_MISSING_TILE, DEVERR_PIXEL_RANGE = 0, 1, 2
ABI_VERSION = 2
POINTING_EXACT, POINTING_CERTIFIED, POINTING_MIXED = 0, 1, 2
HOST_NONE, HOST_MAPPED, HOST_PAGEABLE = 0, 1, 2
LUT_N = 1 << 14

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_void_p = ctypes.c_void_p
c_double = ctypes.c_double


class Pixelization(ctypes.Structure):
    _fields_ = [
        ("coord_sys", c_int32),
        ("pix_sys", c_int32),
        ("tiled", c_int32),
        ("interp", c_int32),
        ("n_comp", c_int32),
        ("naxis", c_int32 * 2),
        ("tile_shape", c_int32 * 2),
        ("nside", c_int32),
        ("nest", c_int32),
        ("nside_tile", c_int32),
        ("pointing", c_int32),
        ("cdelt", c_double * 2),
        ("crpix", c_double * 2),
    ]


class Map(ctypes.Structure):
    _fields_ = [
        ("data", c_void_p),
        ("tile_offset", c_void_p),
        ("n_tile", c_int32),
        ("_pad", c_int32),
    ]


class Ranges(ctypes.Structure):
    _fields_ = [
        ("seg", c_void_p),
        ("n_seg", c_int32),
        ("max_len", c_int32),
    ]


class PrecompGeom(ctypes.Structure):
    _fields_ = [
        ("tiled", c_int32),
        ("n_comp", c_int32),
        ("naxis", c_int32 * 2),
        ("tile_dims", c_void_p),
    ]


class Obs(ctypes.Structure):
    _fields_ = [
        ("boresight", c_void_p),
        ("dets", c_void_p),
        ("response", c_void_p),
        ("signal", c_void_p),
        ("det_weights", c_void_p),
        ("sig_det_stride", c_int64),
        ("n_time", c_int32),
        ("n_det", c_int32),
    ]


class SightLine(ctypes.Structure):
    _fields_ = [
        ("kind", c_int32),
        ("has_left", c_int32),
        ("roll", c_double),
        ("site_lon_rad", c_double),
        ("era_epoch", c_double),
        ("era_poly", c_double * 2),
        ("q_site_lat", c_double * 4),
        ("q_pi", c_double * 4),
        ("q_left", c_double * 4),
    ]


# enum so3g_sight_kind
SIGHT_HORIZON, SIGHT_NAIVE_AZEL = 0, 1

P = ctypes.POINTER
_SIGS = {
    "so3g_init": (ctypes.c_int, []),
    "so3g_last_error": (ctypes.c_char_p, []),
    "so3g_abi_version": (ctypes.c_int, []),
    "so3g_get_trig_tables": (ctypes.c_int, [c_void_p, c_void_p, c_int32]),
    "so3g_launch_count": (c_int64, []),
    "so3g_set_chunked_min_samples": (c_int64, [c_int64]),
    "so3g_host_access": (ctypes.c_int, [c_void_p, c_void_p]),
    "so3g_proj_coords": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p, c_int32,
                                        c_void_p, c_void_p]),
    "so3g_proj_pixels": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p, c_int32,
                                        c_void_p, c_void_p]),
    "so3g_proj_pointing_matrix": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                                 c_int32, c_void_p, c_void_p, c_void_p,
                                                 c_void_p]),
    "so3g_proj_tile_hits": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                           c_int32, c_void_p, c_int32, c_void_p]),
    "so3g_proj_domain_edges": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                              c_int32, c_int32, c_int32, P(Map), c_void_p,
                                              c_int32, c_void_p, c_int64, c_void_p, c_void_p,
                                              c_void_p]),
    "so3g_proj_to_map": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p, c_int32,
                                        c_void_p, c_void_p, c_int64, c_void_p, P(Ranges),
                                        P(Map), c_int32, c_void_p, c_void_p]),
    "so3g_proj_to_map_noalloc": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                                c_int32, c_void_p, c_void_p, c_int64, c_void_p,
                                                c_void_p, c_int32, c_void_p, c_void_p, c_int32,
                                                c_int32, c_void_p, c_void_p]),
    "so3g_noalloc_read_error": (ctypes.c_int, [c_void_p, c_void_p]),
    "so3g_proj_to_weight_map": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                               c_int32, c_void_p, c_void_p, P(Ranges), P(Map),
                                               c_int32, c_void_p, c_void_p]),
    "so3g_proj_from_map": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p, c_int32,
                                          c_void_p, P(Map), c_void_p, c_int64, c_void_p,
                                          c_void_p]),
    "so3g_batch_work_offsets": (c_int64, [P(Obs), c_int32, c_int32, c_void_p]),
    "so3g_proj_to_map_batch": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32, c_void_p,
                                              c_int64, c_int32, c_int32, P(Map), c_int32,
                                              c_void_p, c_void_p]),
    "so3g_proj_to_weight_map_batch": (ctypes.c_int, [P(Pixelization), c_void_p, c_int32,
                                                     c_void_p, c_int64, c_int32, c_int32,
                                                     P(Map), c_int32, c_void_p, c_void_p]),
    "so3g_precomp_to_map": (ctypes.c_int, [P(PrecompGeom), c_void_p, c_void_p, c_int32, c_int32,
                                           c_void_p, c_int64, c_void_p, P(Ranges), P(Map),
                                           c_int32, c_void_p, c_void_p]),
    "so3g_precomp_to_weight_map": (ctypes.c_int, [P(PrecompGeom), c_void_p, c_void_p, c_int32,
                                                  c_int32, c_void_p, P(Ranges), P(Map),
                                                  c_int32, c_void_p, c_void_p]),
    "so3g_precomp_from_map": (ctypes.c_int, [P(PrecompGeom), c_void_p, c_void_p, c_int32,
                                             c_int32, P(Map), c_void_p, c_int64, c_void_p,
                                             c_void_p]),
    "so3g_boresight": (ctypes.c_int, [P(SightLine), c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_int64, c_void_p, c_void_p]),
    "so3g_quat_left_multiply": (ctypes.c_int, [c_void_p, c_void_p, c_int64, c_void_p,
                                               c_void_p]),
    "so3g_mask_count_segments": (ctypes.c_int, [c_void_p, c_int32, c_int32, c_int64, c_void_p,
                                                c_void_p]),
    "so3g_mask_fill_segments": (ctypes.c_int, [c_void_p, c_int32, c_int32, c_int64, c_void_p,
                                               c_void_p, c_void_p, c_void_p, c_void_p]),
}

_lib = None
_lock = threading.Lock()


class LibraryError(RuntimeError):
    """The CUDA library is missing or failed."""


def symbols():
    """Names of the C entry points (all declared in include/so3g_gb300.h)."""
    return list(_SIGS)


def lib():
    """Load libso3g_gb300.so (once) and return the ctypes handle."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise LibraryError(
                "The so3g_gb300 CUDA library is not built (%s is missing). Run "
                "`python -c \"import so3g_gb300.build as b; b.build()\"` (needs nvcc)." % LIB_PATH)
        h = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        if h.so3g_abi_version() != ABI_VERSION:
            raise LibraryError("libso3g_gb300.so ABI version %d, expected %d"
                               % (h.so3g_abi_version(), ABI_VERSION))
        _lib = h
        return _lib


def last_error():
    msg = lib().so3g_last_error()
    return msg.decode() if msg else ""


def check(rc, what):
    """Raise for a negative status from an entry point."""
    if rc == 0:
        return
    msg = last_error()
    if rc == -1:
        raise ValueError("%s: %s" % (what, msg))
    raise LibraryError("%s failed (status %d): %s" % (what, rc, msg))
