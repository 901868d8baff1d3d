// Stand-in for spt3g's container_pybindings.h -- TEST INFRASTRUCTURE for
// oracle/ref_engine.cpp; src/Projection.cxx uses nothing from it.
#pragma once
#include <boost/python.hpp>
