// Boost trim subset (TEST INFRASTRUCTURE): strip leading and trailing white space in place.
#ifndef DFTG_SHIM_BOOST_TRIM
#define DFTG_SHIM_BOOST_TRIM
#include <cctype>
#include <string>
namespace boost {
namespace algorithm {
inline void trim(std::string &s)
{
    size_t b = 0, e = s.size();
    while (b < e && std::isspace((unsigned char)s[b])) ++b;
    while (e > b && std::isspace((unsigned char)s[e - 1])) --e;
    s = s.substr(b, e - b);
}
}  // namespace algorithm
using algorithm::trim;
}  // namespace boost
#endif
