// Boost string-algorithm subset (TEST INFRASTRUCTURE): split with is_any_of
// and token compression, trim.  split keeps a leading empty token when the
// input starts with a delimiter, as Boost does.
#ifndef DFTG_SHIM_BOOST_STRING
#define DFTG_SHIM_BOOST_STRING
#include <cctype>
#include <string>
#include <vector>
#include "string/trim.hpp"
namespace boost {
namespace algorithm {
enum token_compress_mode_type { token_compress_on, token_compress_off };
struct any_of_pred {
    std::string set;
    bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
inline any_of_pred is_any_of(const std::string &s) { return any_of_pred{s}; }
template <typename Pred>
inline std::vector<std::string> &split(std::vector<std::string> &out, const std::string &in, Pred p,
                                       token_compress_mode_type mode = token_compress_off)
{
    out.clear();
    std::string cur;
    size_t i = 0;
    while (true) {
        if (i == in.size()) { out.push_back(cur); break; }
        if (p(in[i])) {
            out.push_back(cur);
            cur.clear();
            ++i;
            if (mode == token_compress_on)
                while (i < in.size() && p(in[i])) ++i;
            continue;
        }
        cur.push_back(in[i++]);
    }
    return out;
}
}  // namespace algorithm
using algorithm::is_any_of;
using algorithm::split;
using algorithm::token_compress_on;
using algorithm::token_compress_off;
}  // namespace boost
#endif
