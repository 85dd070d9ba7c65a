/*
 * Test infrastructure (oracle): stand-in for Boost.Math's bessel.hpp, which
 * is not installed here.  The reference evaluates its Chebyshev weights with
 * boost::math::cyl_bessel_i(k, s) (LightNE/SpectralPropagation.h:8-12), in
 * double for an integer order and a float argument; this forwards to the
 * C++17 special function std::cyl_bessel_i in double.  Nothing in the
 * product includes it.
 */
#pragma once
#include <cmath>

namespace boost {
namespace math {
template <class T1, class T2>
inline double cyl_bessel_i(T1 v, T2 x) {
  return std::cyl_bessel_i(static_cast<double>(v), static_cast<double>(x));
}
}  // namespace math
}  // namespace boost
