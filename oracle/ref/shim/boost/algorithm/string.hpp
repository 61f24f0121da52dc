// boost::algorithm::string stand-in: trim, split on a character set, token compression.
#ifndef MPSXX_REF_BOOST_ALGORITHM_STRING_HPP
#define MPSXX_REF_BOOST_ALGORITHM_STRING_HPP
#include <cctype>
#include <string>
#include <vector>
#include <boost/mpsxx_shim.hpp>
namespace boost {
namespace algorithm {
enum token_compress_mode_type { token_compress_off, token_compress_on };
struct is_any_of {
  std::string set;
  explicit is_any_of(const char* s) : set(s) {}
  bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
inline void trim(std::string& s) {
  std::size_t b = 0, e = s.size();
  while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
  while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
  s = s.substr(b, e - b);
}
template <class Seq>
Seq& split(Seq& out, const std::string& in, const is_any_of& pred,
           token_compress_mode_type mode = token_compress_off) {
  out.clear();
  std::string cur;
  bool last_sep = false;
  for (char c : in) {
    if (pred(c)) {
      if (!(mode == token_compress_on && last_sep)) out.push_back(cur);
      cur.clear();
      last_sep = true;
    } else {
      cur.push_back(c);
      last_sep = false;
    }
  }
  out.push_back(cur);
  return out;
}
}  // namespace algorithm
using algorithm::is_any_of;
using algorithm::split;
using algorithm::token_compress_off;
using algorithm::token_compress_on;
using algorithm::trim;
}  // namespace boost
#endif
