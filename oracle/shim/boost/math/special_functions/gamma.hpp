// Boost.Math gamma header stand-in (TEST INFRASTRUCTURE): included by the
// reference, which evaluates its incomplete gamma function in gamma.cpp.
#ifndef DFTG_SHIM_BOOST_GAMMA
#define DFTG_SHIM_BOOST_GAMMA
#include <cmath>
#include "factorials.hpp"
#endif
