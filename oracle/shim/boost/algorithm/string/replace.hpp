// Include stand-in for boost/algorithm/string/replace.hpp (boost is not
// installed here): the one algorithm the reference's OBJ material loader
// calls, replace_all(text, search, format) -- every occurrence of `search`
// in `text`, left to right, replaced by `format`.
#pragma once
#include <string>

namespace boost::algorithm {
inline void replace_all(std::string& text, std::string const& search, std::string const& format) {
  if (search.empty()) return;
  std::string out;
  size_t at = 0;
  for (;;) {
    size_t const hit = text.find(search, at);
    if (hit == std::string::npos) break;
    out.append(text, at, hit - at);
    out += format;
    at = hit + search.size();
  }
  out.append(text, at, std::string::npos);
  text.swap(out);
}
}  // namespace boost::algorithm
