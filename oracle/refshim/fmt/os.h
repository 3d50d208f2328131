#pragma once
#include <string>
#include "core.h"
namespace fmt {
struct ostream {
  FILE* f;
  template <class... A> void print(const char* s, const A&... a) { if (f) fputs(format(s, a...).c_str(), f); }
  void close() { if (f) fclose(f); f = nullptr; }
};
inline ostream output_file(const char* name) { return ostream{fopen(name, "w")}; }
inline ostream output_file(const std::string& name) { return ostream{fopen(name.c_str(), "w")}; }
}  // namespace fmt
