// Boost.Regex subset (TEST INFRASTRUCTURE) on top of <regex>.
#ifndef DFTG_SHIM_BOOST_REGEX
#define DFTG_SHIM_BOOST_REGEX
#include <regex>
#include <string>
namespace boost {
typedef std::regex regex;
typedef std::smatch smatch;
using std::regex_match;
}  // namespace boost
#endif
