// Boost.Math binomial header stand-in (TEST INFRASTRUCTURE): the reference
// includes it but forms its binomials from factorials itself.
#ifndef DFTG_SHIM_BOOST_BINOMIAL
#define DFTG_SHIM_BOOST_BINOMIAL
#include "factorials.hpp"
#endif
