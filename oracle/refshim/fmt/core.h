// Minimal stand-in for the {fmt} calls of the reference hot path: each "{...}"
// placeholder takes the next argument (format specs are ignored).
#pragma once
#include <cstdio>
#include <sstream>
#include <string>
namespace fmt {
inline void cdxref_fmt(std::ostringstream& o, const char* f) { o << f; }
template <class A, class... R>
void cdxref_fmt(std::ostringstream& o, const char* f, const A& a, const R&... r) {
  for (; *f; ++f) {
    if (*f == '{' && f[1] != '{') {
      while (*f && *f != '}') ++f;
      o << a;
      if (*f) ++f;
      cdxref_fmt(o, f, r...);
      return;
    }
    o << *f;
  }
}
template <class... A> std::string format(const char* f, const A&... a) {
  std::ostringstream o; cdxref_fmt(o, f, a...); return o.str(); }
template <class... A> void print(const char* f, const A&... a) { fputs(format(f, a...).c_str(), stdout); }
template <class... A> void print(FILE* fp, const char* f, const A&... a) { fputs(format(f, a...).c_str(), fp); }
template <class... A> void println(const char* f, const A&... a) { puts(format(f, a...).c_str()); }
template <class... A> void println(FILE* fp, const char* f, const A&... a) {
  fputs(format(f, a...).c_str(), fp); fputc('\n', fp); }
}  // namespace fmt
