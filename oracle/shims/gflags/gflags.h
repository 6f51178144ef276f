// Shim for gflags: flags are plain globals in the declaring namespace.
#pragma once
#include <cstdint>
#include <string>
#define DEFINE_int32(name, value, help) int32_t FLAGS_##name = value
#define DEFINE_int64(name, value, help) int64_t FLAGS_##name = value
#define DEFINE_uint64(name, value, help) uint64_t FLAGS_##name = value
#define DEFINE_double(name, value, help) double FLAGS_##name = value
#define DEFINE_bool(name, value, help) bool FLAGS_##name = value
#define DEFINE_string(name, value, help) std::string FLAGS_##name = value
#define DECLARE_int32(name) extern int32_t FLAGS_##name
#define DECLARE_int64(name) extern int64_t FLAGS_##name
#define DECLARE_uint64(name) extern uint64_t FLAGS_##name
#define DECLARE_double(name) extern double FLAGS_##name
#define DECLARE_bool(name) extern bool FLAGS_##name
#define DECLARE_string(name) extern std::string FLAGS_##name
namespace gflags {
inline void ParseCommandLineFlags(int*, char***, bool) {}
}  // namespace gflags
