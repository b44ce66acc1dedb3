// Boost lexical_cast subset (TEST INFRASTRUCTURE): string -> number with the
// whole string consumed, otherwise bad_lexical_cast (a std::bad_cast).
#ifndef DFTG_SHIM_BOOST_LEXICAL_CAST
#define DFTG_SHIM_BOOST_LEXICAL_CAST
#include <cerrno>
#include <cstdlib>
#include <string>
#include <typeinfo>
namespace boost {
class bad_lexical_cast : public std::bad_cast {
public:
    const char *what() const noexcept override { return "bad lexical cast"; }
};
namespace shim_detail {
inline void require_all(const std::string &s, const char *end)
{
    if (s.empty() || end != s.c_str() + s.size() || errno == ERANGE) throw bad_lexical_cast();
}
template <typename T> struct caster;
template <> struct caster<double> {
    static double go(const std::string &s) { errno = 0; char *e = nullptr; double v = std::strtod(s.c_str(), &e); require_all(s, e); return v; }
};
template <> struct caster<float> {
    static float go(const std::string &s) { return (float)caster<double>::go(s); }
};
template <> struct caster<unsigned int> {
    static unsigned int go(const std::string &s)
    {
        if (!s.empty() && s[0] == '-') throw bad_lexical_cast();
        errno = 0; char *e = nullptr; unsigned long v = std::strtoul(s.c_str(), &e, 10); require_all(s, e);
        if (v > 0xffffffffUL) throw bad_lexical_cast();
        return (unsigned int)v;
    }
};
template <> struct caster<int> {
    static int go(const std::string &s) { errno = 0; char *e = nullptr; long v = std::strtol(s.c_str(), &e, 10); require_all(s, e); return (int)v; }
};
template <> struct caster<std::string> {
    static std::string go(const std::string &s) { return s; }
};
}  // namespace shim_detail
template <typename T>
inline T lexical_cast(const std::string &s) { return shim_detail::caster<T>::go(s); }
template <typename T>
inline T lexical_cast(const char *s) { return shim_detail::caster<T>::go(std::string(s)); }
}  // namespace boost
#endif
