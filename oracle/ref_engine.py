"""The reference's own ProjectionEngine, compiled from so3g's
src/Projection.cxx in the reference checkout (oracle/ref_engine.cpp,
oracle/refstub) -- TEST INFRASTRUCTURE, used only to check the oracle.

``RefEngine(name, pix_args)`` mirrors a so3g ProjEng_* object: its
methods take and return the same Python objects as so3g's binding (numpy
arrays, lists of per-detector rows, tuples), run the reference's C++ with
the GIL held, and raise the reference's exception classes and messages.
thread_intervals must be None.  Available only where the reference
checkout is (``available()``); nothing on the GPU machine uses it.
"""
import ctypes

from . import build as _build

_lib = None


def _load():
    global _lib
    if _lib is None:
        path = _build.build_ref_engine()
        if path is None:
            raise RuntimeError("the so3g reference checkout is not available")
        lib = ctypes.PyDLL(path)
        lib.ref_engine_init.restype = ctypes.c_int
        if lib.ref_engine_init() != 0:
            raise RuntimeError("numpy C-API initialisation failed")
        lib.ref_engine_call.restype = ctypes.py_object
        lib.ref_engine_call.argtypes = [ctypes.c_char_p, ctypes.py_object, ctypes.c_char_p,
                                        ctypes.py_object]
        _lib = lib
    return _lib


def available():
    return _build.ref_sources_present()


class RefEngine:
    """A ProjEng_* (or ProjEng_Precomp_*) class of the reference."""

    def __init__(self, name, pix_args=None):
        self.name = name
        self.pix_args = pix_args
        self._lib = _load()
        if pix_args is not None:
            self._call("comp_count")      # constructs it: raises on bad args

    def _call(self, method, *args):
        return self._lib.ref_engine_call(self.name.encode(), self.pix_args, method.encode(),
                                         tuple(args))

    @property
    def index_count(self):
        return self._call("index_count")

    @property
    def comp_count(self):
        return self._call("comp_count")

    def __getattr__(self, method):
        if method.startswith("_"):
            raise AttributeError(method)
        return lambda *args: self._call(method, *args)
