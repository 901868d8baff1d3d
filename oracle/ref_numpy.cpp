// ref_numpy.cpp -- TEST INFRASTRUCTURE: holds numpy's C-API table for the
// reference build of oracle/ref_engine.cpp (src/Projection.cxx declares it
// with NO_IMPORT_ARRAY under the name include/so3g_numpy.h gives it) and
// fills it.  ref_engine_init() must run once, with the GIL, before any
// engine call.
#define NPY_API_SYMBOL_ATTRIBUTE
#define PY_ARRAY_UNIQUE_SYMBOL Py_Array_API_SO3G
#define NPY_NO_DEPRECATED_API NPY_1_7_API_VERSION
#include <Python.h>
#include <numpy/arrayobject.h>

extern "C" int ref_engine_init(void) { return _import_array() < 0 ? -1 : 0; }
