// Stand-in for the part of boost.python that so3g's src/Projection.cxx
// uses -- TEST INFRASTRUCTURE for oracle/ref_engine.cpp, which compiles
// the reference's ProjectionEngine from its own source so the oracle can
// be checked against it.  Objects are real CPython objects (new
// references, released on destruction); extract<> converts the few C++
// types the engine reads; class_<> and init<> accept the module
// registration block and do nothing (that block is never run).  Not a
// general boost.python.
#pragma once

#include <Python.h>

#include <string>
#include <type_traits>
#include <utility>

namespace boost {
namespace python {

// A Python error is set; the caller unwinds to the wrapper, which returns
// NULL to Python.
struct error_already_set {};
inline void throw_error_already_set() { throw error_already_set(); }

template <class T = PyObject>
struct handle {
    PyObject *p;   // a new reference, or NULL (an error is set)
    explicit handle(PyObject *x) : p(x) {}
};

class object;
// C++ values the engine wraps in an object: integers, floats and (through
// to_python, found by argument-dependent lookup) the reference's Ranges.
inline PyObject *to_python(long v) { return PyLong_FromLong(v); }
inline PyObject *to_python(int v) { return PyLong_FromLong(v); }
inline PyObject *to_python(double v) { return PyFloat_FromDouble(v); }

class object {
public:
    object() : p_(Py_None) { Py_INCREF(p_); }
    template <class T>
    explicit object(const handle<T> &h) : p_(h.p) {
        if (!p_) throw error_already_set();
    }
    object(const object &o) : p_(o.p_) { Py_INCREF(p_); }
    object(object &&o) noexcept : p_(o.p_) { o.p_ = nullptr; }
    template <class T, class = typename std::enable_if<
                           !std::is_base_of<object, typename std::decay<T>::type>::value>::type>
    explicit object(const T &v) : p_(to_python(v)) {
        if (!p_) throw error_already_set();
    }
    object &operator=(const object &o) {
        Py_INCREF(o.p_);
        Py_XDECREF(p_);
        p_ = o.p_;
        return *this;
    }
    ~object() { Py_XDECREF(p_); }

    PyObject *ptr() const { return p_; }
    // A new reference for the caller.
    PyObject *release() {
        PyObject *r = p_;
        p_ = nullptr;
        return r;
    }
    static object borrowed(PyObject *p) {
        Py_INCREF(p);
        return object(handle<>(p));
    }

    object operator[](long i) const {
        return object(handle<>(PySequence_GetItem(p_, (Py_ssize_t)i)));
    }
    object attr(const char *name) const {
        return object(handle<>(PyObject_GetAttrString(p_, name)));
    }
    object operator()() const { return object(handle<>(PyObject_CallNoArgs(p_))); }

protected:
    PyObject *p_;
};

inline long len(const object &o) {
    const Py_ssize_t n = PyObject_Length(o.ptr());
    if (n < 0) throw error_already_set();
    return (long)n;
}

class list : public object {
public:
    list() : object(handle<>(PyList_New(0))) {}
    explicit list(const object &o) : object(o) {}
    template <class X>
    void append(const X &x) {
        const object v(x);
        if (PyList_Append(p_, v.ptr()) < 0) throw error_already_set();
    }
    void append(const object &v) {
        if (PyList_Append(p_, v.ptr()) < 0) throw error_already_set();
    }
};

class tuple : public object {
public:
    tuple() : object(handle<>(PyTuple_New(0))) {}
    explicit tuple(const object &o) : object(o) {}
};

template <class A, class B>
tuple make_tuple(const A &a, const B &b) {
    const object oa(a), ob(b);
    return tuple(object(handle<>(PyTuple_Pack(2, oa.ptr(), ob.ptr()))));
}

// extract<T>(o): check() says whether o converts to T; operator() and the
// conversion operator convert (raising on failure).  Types the engine
// does not convert from Python (e.g. its Ranges) never check.
template <class T>
struct extract {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return false; }
    T operator()() const {
        PyErr_SetString(PyExc_TypeError, "unsupported conversion in the reference build");
        throw error_already_set();
    }
    operator T() const { return (*this)(); }
};

template <>
struct extract<object> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return true; }
    object operator()() const { return o; }
    operator object() const { return o; }
};

template <>
struct extract<list> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return PyList_Check(o.ptr()); }
    list operator()() const {
        if (!check()) {
            PyErr_SetString(PyExc_TypeError, "expected a list");
            throw error_already_set();
        }
        return list(o);
    }
    operator list() const { return (*this)(); }
};

template <>
struct extract<tuple> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return PyTuple_Check(o.ptr()); }
    tuple operator()() const {
        if (!check()) {
            PyErr_SetString(PyExc_TypeError, "expected a tuple");
            throw error_already_set();
        }
        return tuple(o);
    }
    operator tuple() const { return (*this)(); }
};

template <>
struct extract<int> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return PyLong_Check(o.ptr()) && !PyBool_Check(o.ptr()); }
    int operator()() const {
        const long v = PyLong_AsLong(o.ptr());
        if (v == -1 && PyErr_Occurred()) throw error_already_set();
        return (int)v;
    }
    operator int() const { return (*this)(); }
};

template <>
struct extract<bool> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return PyBool_Check(o.ptr()) || PyLong_Check(o.ptr()); }
    bool operator()() const {
        const int v = PyObject_IsTrue(o.ptr());
        if (v < 0) throw error_already_set();
        return v != 0;
    }
    operator bool() const { return (*this)(); }
};

template <>
struct extract<double> {
    object o;
    explicit extract(const object &x) : o(x) {}
    bool check() const { return PyFloat_Check(o.ptr()) || PyLong_Check(o.ptr()); }
    double operator()() const {
        const double v = PyFloat_AsDouble(o.ptr());
        if (v == -1.0 && PyErr_Occurred()) throw error_already_set();
        return v;
    }
    operator double() const { return (*this)(); }
};

// Registration: accepted and ignored.
template <class... T>
struct init {};

template <class W, class... X>
struct class_ {
    template <class... A>
    explicit class_(A &&...) {}
    template <class... A>
    class_ &def(A &&...) { return *this; }
    template <class... A>
    class_ &add_property(A &&...) { return *this; }
};

}  // namespace python
}  // namespace boost
