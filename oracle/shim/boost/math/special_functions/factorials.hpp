// Boost.Math factorial subset for building the reference's translation units
// here (TEST INFRASTRUCTURE; Boost is not installed in this image).
// factorial<T>(n) = n!, double_factorial<T>(n) = n!! as floating-point
// products in ascending order; exact in double while the value needs at most
// 53 significant bits (every n! up to 22!).
#ifndef DFTG_SHIM_BOOST_FACTORIALS
#define DFTG_SHIM_BOOST_FACTORIALS
// Boost's header brings in the standard containers its tables use; the
// reference relies on that for std::vector.
#include <vector>
namespace boost {
namespace math {
template <typename T>
inline T factorial(unsigned n)
{
    T f = T(1);
    for (unsigned k = 2; k <= n; ++k) f *= T(k);
    return f;
}
template <typename T>
inline T double_factorial(unsigned n)
{
    T f = T(1);
    for (unsigned k = n; k > 1; k -= 2) f *= T(k);
    return f;
}
}  // namespace math
}  // namespace boost
#endif
