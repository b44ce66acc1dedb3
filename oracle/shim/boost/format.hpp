// Boost.Format subset (TEST INFRASTRUCTURE): printf-style directives filled
// by operator% in order and written by operator<<.  Integral arguments are
// printed with the directive's flags and width as integers, floating-point
// ones with the directive as given (or %g when it names an integer), strings
// with %s; "%%" is a literal percent sign.
#ifndef DFTG_SHIM_BOOST_FORMAT
#define DFTG_SHIM_BOOST_FORMAT
#include <cstdio>
#include <ostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <vector>

namespace boost {

class format {
public:
    explicit format(const std::string &f) { parse(f); }
    explicit format(const char *f) { parse(f); }

    template <typename T>
    format &operator%(const T &v)
    {
        if (next_ < specs_.size()) values_[next_] = render(specs_[next_], v);
        ++next_;
        return *this;
    }

    std::string str() const
    {
        std::string out;
        for (size_t i = 0; i < text_.size(); ++i) {
            out += text_[i];
            if (i < specs_.size()) out += values_[i];
        }
        return out;
    }

private:
    void parse(const std::string &f)
    {
        std::string cur;
        size_t i = 0;
        while (i < f.size()) {
            if (f[i] != '%') { cur.push_back(f[i++]); continue; }
            if (i + 1 < f.size() && f[i + 1] == '%') { cur.push_back('%'); i += 2; continue; }
            size_t j = i + 1;
            while (j < f.size() && std::string("0123456789.+- #").find(f[j]) != std::string::npos) ++j;
            if (j < f.size()) ++j;   // conversion character
            text_.push_back(cur);
            cur.clear();
            specs_.push_back(f.substr(i, j - i));
            i = j;
        }
        text_.push_back(cur);
        values_.assign(specs_.size(), std::string());
    }

    template <typename T>
    static std::string render(const std::string &spec, const T &v)
    {
        char buf[128];
        const std::string flags = spec.substr(0, spec.size() - 1);
        const char conv = spec.empty() ? 's' : spec.back();
        if constexpr (std::is_integral<T>::value) {
            std::string f = flags;
            const size_t dot = f.find('.');
            if (dot != std::string::npos) f = f.substr(0, dot);
            f += std::is_signed<T>::value ? "lld" : "llu";
            if (std::is_signed<T>::value) std::snprintf(buf, sizeof buf, f.c_str(), (long long)v);
            else std::snprintf(buf, sizeof buf, f.c_str(), (unsigned long long)v);
            return buf;
        } else if constexpr (std::is_floating_point<T>::value) {
            const std::string f = std::string("eEfFgG").find(conv) != std::string::npos ? spec : std::string("%g");
            std::snprintf(buf, sizeof buf, f.c_str(), (double)v);
            return buf;
        } else {
            std::ostringstream os;
            os << v;
            return os.str();
        }
    }

    std::vector<std::string> text_, specs_, values_;
    size_t next_ = 0;
};

inline std::ostream &operator<<(std::ostream &os, const format &f) { return os << f.str(); }

}  // namespace boost
#endif
