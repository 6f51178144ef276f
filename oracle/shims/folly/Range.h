// Shim for folly::StringPiece (a non-owning string view with hash()).
#pragma once
#include <cstddef>
#include <cstring>
#include <functional>
#include <string>
namespace folly {
class StringPiece {
 public:
  StringPiece() : b_(nullptr), n_(0) {}
  StringPiece(const char* s) : b_(s), n_(s ? std::strlen(s) : 0) {}
  StringPiece(const char* s, std::size_t n) : b_(s), n_(n) {}
  StringPiece(const std::string& s) : b_(s.data()), n_(s.size()) {}
  const char* data() const { return b_; }
  const char* begin() const { return b_; }
  const char* end() const { return b_ + n_; }
  std::size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  std::string str() const { return std::string(b_, n_); }
  std::string toString() const { return str(); }
  std::size_t hash() const { return std::hash<std::string>()(str()); }
  char operator[](std::size_t i) const { return b_[i]; }
  bool operator==(const StringPiece& o) const { return n_ == o.n_ && std::memcmp(b_, o.b_, n_) == 0; }
 private:
  const char* b_;
  std::size_t n_;
};
}  // namespace folly
