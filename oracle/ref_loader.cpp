// ref_loader.cpp -- the reference's text loader as a test checker.
//
// TEST INFRASTRUCTURE ONLY: compiles the reference's main/main.cpp (its
// LoadData, main/main.cpp:49-109, lives in an anonymous namespace there, so
// the file is included into this translation unit) against the shims under
// oracle/shims, and exposes LoadData through a C entry point.  The
// reference's main() is renamed and never called; its configuration class is
// only declared by the reference headers and gets a stub here.
#define main qfref_reference_main_unused
#include "main/main.cpp"
#undef main

#include <cstring>

quickfoil::Configuration::Configuration(const std::string&) { std::abort(); }

extern "C" {

// Loads a '|'-delimited file as the reference does: num_args arguments per
// line, skipped[i] nonzero for an argument the configuration skips.  Writes
// the kept columns (capacity rows each) and the row count; returns 0, or 1
// when capacity is too small (num_rows still holds the count).  Lines the
// reference rejects abort the process (its CHECK / LOG(FATAL)).
int qfref_load_text(const char* path, int num_args, const int* skipped, int32_t* const* out,
                    int64_t capacity, int64_t* num_rows) {
  quickfoil::Vector<quickfoil::PredicateArgumentConfiguration> args;
  for (int i = 0; i < num_args; ++i) args.emplace_back(0, skipped != nullptr && skipped[i] != 0);
  quickfoil::PredicateConfiguration conf("loaded", path, std::move(args), -1);
  quickfoil::Vector<quickfoil::ConstBufferPtr> blocks;
  quickfoil::LoadData(conf, path, &blocks);
  const int64_t n = blocks.empty() ? 0 : (int64_t)blocks[0]->num_tuples();
  *num_rows = n;
  if (n > capacity) return 1;
  for (size_t c = 0; c < blocks.size(); ++c)
    if (n > 0) memcpy(out[c], blocks[c]->as_type<int32_t>(), sizeof(int32_t) * (size_t)n);
  return 0;
}

}  // extern "C"
