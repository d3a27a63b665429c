// Test infrastructure only: a minimal stand-in for the one Boost string
// routine the reference host code calls (src/input.hpp:90-110 uses
// boost::split with boost::is_space() and token_compress_on).  Semantics
// follow Boost's documented behaviour: separator runs collapse to one split
// point when compression is on; a leading (trailing) separator run yields one
// empty leading (trailing) token; an empty input yields one empty token.
#ifndef LBFFS_BOOST_STUB_STRING_HPP
#define LBFFS_BOOST_STUB_STRING_HPP
#include <algorithm>
#include <cctype>
#include <string>
#include <vector>

namespace boost {
namespace algorithm {
enum token_compress_mode_type { token_compress_on, token_compress_off };
}  // namespace algorithm

struct is_space_pred {
    bool operator()(char c) const { return std::isspace(static_cast<unsigned char>(c)) != 0; }
};
inline is_space_pred is_space() { return is_space_pred(); }

template <class Pred>
std::vector<std::string>& split(std::vector<std::string>& out, const std::string& in, Pred sep,
                                algorithm::token_compress_mode_type mode = algorithm::token_compress_off)
{
    out.clear();
    std::string tok;
    std::size_t i = 0, n = in.size();
    for (;;) {
        if (i == n) {
            out.push_back(tok);
            break;
        }
        if (sep(in[i])) {
            out.push_back(tok);
            tok.clear();
            ++i;
            if (mode == algorithm::token_compress_on)
                while (i < n && sep(in[i])) ++i;
        } else {
            tok.push_back(in[i++]);
        }
    }
    return out;
}
}  // namespace boost
#endif
