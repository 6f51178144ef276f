// Shim for boost::split / boost::is_any_of as main/main.cpp uses them:
// split a string at every character of a set, keeping empty fields (the
// documented behaviour of boost::split without token compression).
#pragma once
#include <string>
#include <vector>
namespace boost {
struct qfshim_any_of {
  std::string set;
  bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
inline qfshim_any_of is_any_of(const char* s) { return qfshim_any_of{s}; }
inline std::vector<std::string>& split(std::vector<std::string>& out, const std::string& in,
                                       const qfshim_any_of& pred) {
  out.clear();
  std::string cur;
  for (char c : in) {
    if (pred(c)) {
      out.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(c);
    }
  }
  out.push_back(cur);
  return out;
}
}  // namespace boost
