// Stand-in for spt3g's pybindings.h as so3g's src/Projection.cxx uses it --
// TEST INFRASTRUCTURE for oracle/ref_engine.cpp: the module registration
// block PYBINDINGS("so3g") { ... } becomes an ordinary function that is
// compiled (instantiating every engine method it names) but never run.
#pragma once

#include <Python.h>
#include <boost/python.hpp>

// The standard headers and the namespace alias that spt3g's pybindings.h
// and the real boost.python headers make visible to the files that
// include them.
#include <algorithm>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

namespace bp = boost::python;

#define PYBINDINGS(name) void so3g_ref_unused_registration()
