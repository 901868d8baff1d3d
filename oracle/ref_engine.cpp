// ref_engine.cpp -- TEST INFRASTRUCTURE: the reference's own
// ProjectionEngine (so3g src/Projection.cxx, with include/so_linterp.h and
// src/healpix_bare.c), compiled from its source in the reference checkout
// against the stand-in headers of oracle/refstub (boost.python over real
// CPython objects, boost's quaternion, spt3g's binding macros), so that
// the oracle (oracle/proj_oracle.cpp) can be checked against it.
//
// One entry point, ref_engine_call(class name, pixelizor args, method,
// args tuple), loaded with ctypes.PyDLL (the GIL is held, as the
// reference's binding holds it): it builds the named ProjEng_* class and
// calls the method with the given Python objects, returning its Python
// result, or NULL with the reference's exception class and message set.
//
// Differences from the reference's build, all outside the arithmetic:
// - thread_intervals must be None (the reference's Ranges converters are
//   not built); pixel_ranges and tile_ranges return each Ranges as
//   (count, [(start, end), ...]);
// - the two Ranges members Projection.cxx calls (defined in the
//   reference's Ranges.cxx, which is not compiled) are defined below;
// - compiled with -DNDEBUG, so derive_ranges' assert on an unrecognised
//   thread_intervals cannot abort the interpreter.

#include "Projection.cxx"

#include <functional>
#include <map>

// Ranges<T> members used by Projection.cxx (pixel_ranges, tile_ranges,
// derive_ranges): append without checks; insert keeping the intervals
// sorted, then merge those that overlap or touch.
template <typename T>
Ranges<T> &Ranges<T>::append_interval_no_check(const T start, const T end) {
    segments.push_back(std::make_pair(start, end));
    return *this;
}

template <typename T>
Ranges<T> &Ranges<T>::add_interval(const T start, const T end) {
    auto at = std::lower_bound(segments.begin(), segments.end(), std::make_pair(start, end));
    segments.insert(at, std::make_pair(start, end));
    std::vector<std::pair<T, T>> merged;
    for (const auto &s : segments) {
        if (!merged.empty() && s.first <= merged.back().second)
            merged.back().second = std::max(merged.back().second, s.second);
        else
            merged.push_back(s);
    }
    segments.swap(merged);
    return *this;
}

// A Ranges as a Python object: (count, [(start, end), ...]).
PyObject *to_python(const Ranges<int32_t> &r) {
    PyObject *iv = PyList_New((Py_ssize_t)r.segments.size());
    if (!iv) return nullptr;
    for (size_t i = 0; i < r.segments.size(); i++)
        PyList_SET_ITEM(iv, (Py_ssize_t)i,
                        Py_BuildValue("(ii)", r.segments[i].first, r.segments[i].second));
    PyObject *out = Py_BuildValue("(iN)", (int)r.count, iv);
    return out;
}

namespace {

using Call = std::function<bp::object(PyObject *, const std::string &, PyObject *)>;

bp::object arg(PyObject *args, Py_ssize_t i) {
    if (i >= PyTuple_GET_SIZE(args)) {
        PyErr_Format(PyExc_TypeError, "missing argument %zd", i);
        throw bp::error_already_set();
    }
    return bp::object::borrowed(PyTuple_GET_ITEM(args, i));
}

int int_arg(PyObject *args, Py_ssize_t i) {
    return bp::extract<int>(arg(args, i))();
}

template <class E>
bp::object call_engine(PyObject *pix, const std::string &m, PyObject *a) {
    E eng(bp::object::borrowed(pix));
    if (m == "index_count") return bp::object(eng.index_count());
    if (m == "comp_count") return bp::object(eng.comp_count());
    if (m == "coords") return eng.coords(arg(a, 0), arg(a, 1), arg(a, 2));
    if (m == "pixels") return eng.pixels(arg(a, 0), arg(a, 1), arg(a, 2));
    if (m == "pointing_matrix")
        return eng.pointing_matrix(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4));
    if (m == "pixel_ranges")
        return eng.pixel_ranges(arg(a, 0), arg(a, 1), arg(a, 2), int_arg(a, 3));
    if (m == "tile_hits") {
        const std::vector<int> h = eng.tile_hits(arg(a, 0), arg(a, 1));
        bp::list out;
        for (int v : h) out.append(bp::object(v));
        return out;
    }
    if (m == "tile_ranges") return eng.tile_ranges(arg(a, 0), arg(a, 1), arg(a, 2));
    if (m == "zeros") return eng.zeros(arg(a, 0));
    if (m == "from_map")
        return eng.from_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4));
    if (m == "to_map")
        return eng.to_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4), arg(a, 5),
                          arg(a, 6));
    if (m == "to_weight_map")
        return eng.to_weight_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4),
                                 arg(a, 5));
    PyErr_Format(PyExc_AttributeError, "no method %s", m.c_str());
    throw bp::error_already_set();
}

template <class E>
bp::object call_precomp(PyObject *, const std::string &m, PyObject *a) {
    E eng;
    if (m == "from_map") return eng.from_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3));
    if (m == "to_map")
        return eng.to_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4), arg(a, 5));
    if (m == "to_weight_map")
        return eng.to_weight_map(arg(a, 0), arg(a, 1), arg(a, 2), arg(a, 3), arg(a, 4));
    PyErr_Format(PyExc_AttributeError, "no method %s", m.c_str());
    throw bp::error_already_set();
}

#define REF_ONE(N) {#N, &call_engine<N>},
#define REF_TILING(PIX, S, TILING) REF_ONE(ProjEng_##PIX##_##S##_##TILING) \
    REF_ONE(ProjEng_##PIX##_##S##_##TILING##_Bilinear)
#define REF_SPIN(PIX, S) REF_TILING(PIX, S, Tiled) REF_TILING(PIX, S, NonTiled)
#define REF_PIX(PIX) REF_SPIN(PIX, T) REF_SPIN(PIX, QU) REF_SPIN(PIX, TQU)

const std::map<std::string, Call> &engines() {
    static const std::map<std::string, Call> table = {
        REF_PIX(Flat) REF_PIX(Quat) REF_PIX(CAR) REF_PIX(CEA) REF_PIX(ARC) REF_PIX(SIN)
        REF_PIX(TAN) REF_PIX(ZEA)
        REF_ONE(ProjEng_HP_T_NonTiled) REF_ONE(ProjEng_HP_QU_NonTiled)
        REF_ONE(ProjEng_HP_TQU_NonTiled) REF_ONE(ProjEng_HP_T_Tiled)
        REF_ONE(ProjEng_HP_QU_Tiled) REF_ONE(ProjEng_HP_TQU_Tiled)
        {"ProjEng_Precomp_NonTiled", &call_precomp<ProjEng_Precomp_NonTiled>},
        {"ProjEng_Precomp_Tiled", &call_precomp<ProjEng_Precomp_Tiled>},
    };
    return table;
}

}  // namespace

extern "C" PyObject *ref_engine_call(const char *name, PyObject *pix, const char *method,
                                     PyObject *args) {
    try {
        if (!PyTuple_Check(args)) {
            PyErr_SetString(PyExc_TypeError, "args must be a tuple");
            return nullptr;
        }
        const auto &t = engines();
        const auto it = t.find(name);
        if (it == t.end()) {
            PyErr_Format(PyExc_AttributeError, "no engine %s", name);
            return nullptr;
        }
        return it->second(pix, method, args).release();
    } catch (bp::error_already_set &) {
        return nullptr;
    } catch (ValueError_exception &e) {
        PyErr_SetString(PyExc_ValueError, e.msg_for_python().c_str());
    } catch (TypeError_exception &e) {
        PyErr_SetString(PyExc_TypeError, e.msg_for_python().c_str());
    } catch (RuntimeError_exception &e) {
        PyErr_SetString(PyExc_RuntimeError, e.msg_for_python().c_str());
    } catch (so3g_exception &e) {
        PyErr_SetString(PyExc_RuntimeError, e.msg_for_python().c_str());
    } catch (std::exception &e) {
        PyErr_SetString(PyExc_RuntimeError, e.what());
    }
    return nullptr;
}
