// Shim for folly::dynamic: the loader checker compiles the reference's
// main/main.cpp, whose configuration header names the type; the JSON
// configuration itself is never read.
#pragma once
namespace folly {
struct dynamic {};
}  // namespace folly
