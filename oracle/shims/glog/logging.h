// Shim for glog, for compiling the reference's sources as a test checker.
// LOG(FATAL) and CHECK failures print and abort; other logging is dropped;
// DCHECKs compile away as in the reference's release build (NDEBUG).
#pragma once
#include <cstdlib>
#include <iostream>
#include <sstream>

namespace qfshim {
struct NullStream {
  template <typename T>
  NullStream& operator<<(const T&) { return *this; }
  NullStream& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};
struct FatalStream {
  std::ostringstream os;
  FatalStream(const char* file, int line) { os << file << ":" << line << ": "; }
  ~FatalStream() {
    std::cerr << os.str() << std::endl;
    std::abort();
  }
  template <typename T>
  FatalStream& operator<<(const T& v) { os << v; return *this; }
  FatalStream& operator<<(std::ostream& (*f)(std::ostream&)) { os << f; return *this; }
};
}  // namespace qfshim

#define QFSHIM_LOG_INFO qfshim::NullStream()
#define QFSHIM_LOG_WARNING qfshim::NullStream()
#define QFSHIM_LOG_ERROR qfshim::NullStream()
#define QFSHIM_LOG_FATAL qfshim::FatalStream(__FILE__, __LINE__)
#define LOG(severity) QFSHIM_LOG_##severity
#define VLOG(level) qfshim::NullStream()
#define DVLOG(level) qfshim::NullStream()
#define VLOG_IS_ON(level) false
#define CHECK(cond) \
  if (cond) {       \
  } else            \
    qfshim::FatalStream(__FILE__, __LINE__) << "Check failed: " #cond " "
#define CHECK_EQ(a, b) CHECK((a) == (b))
#define CHECK_NE(a, b) CHECK((a) != (b))
#define CHECK_LT(a, b) CHECK((a) < (b))
#define CHECK_LE(a, b) CHECK((a) <= (b))
#define CHECK_GT(a, b) CHECK((a) > (b))
#define CHECK_GE(a, b) CHECK((a) >= (b))
#define CHECK_NOTNULL(p) (p)
#define DCHECK(cond) while (false) qfshim::NullStream()
#define DCHECK_EQ(a, b) while (false) qfshim::NullStream()
#define DCHECK_NE(a, b) while (false) qfshim::NullStream()
#define DCHECK_LT(a, b) while (false) qfshim::NullStream()
#define DCHECK_LE(a, b) while (false) qfshim::NullStream()
#define DCHECK_GT(a, b) while (false) qfshim::NullStream()
#define DCHECK_GE(a, b) while (false) qfshim::NullStream()
#define DLOG(severity) qfshim::NullStream()
#define LOG_IF(severity, cond) qfshim::NullStream()
#define DLOG_IF(severity, cond) qfshim::NullStream()
namespace google {
inline void InitGoogleLogging(const char*) {}
}  // namespace google
static int FLAGS_v = 0;
