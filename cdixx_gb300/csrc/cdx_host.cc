// Host-side pieces of the CDI path: the algorithm-string parser, .bin image
// I/O and the per-thread error string.  No CUDA here.
#include "cdx_host.h"

#include <cctype>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace cdx {

// Fixed per-thread buffer: recording an error never allocates.
static thread_local char g_err[512];

int set_error_cstr(int code, const char* msg) {
  snprintf(g_err, sizeof g_err, "%s", msg ? msg : "");
  return code;
}
int set_error(int code, const std::string& msg) { return set_error_cstr(code, msg.c_str()); }
const char* last_error() { return g_err; }

// ------------------------------------------------------------------ AlgoParser
// Grammar of AlgoParser (src/independant/readConfig.cc:82-163):
//   expr := term ('+' term)*     term := count '*' (NAME | '(' expr ')')
// blanks ignored, NAME one of the Algorithm enum spellings (readConfig.cc:121-131),
// `n*X` repeating X n times in order.  The reference cuts a parenthesised group
// at the first ')' and therefore rejects nested groups; here they nest.  A
// count of 0 after the first term of a group makes the reference's next() repeat that
// step forever (its counter goes negative); such strings are rejected.
namespace {
struct Parser {
  const std::string& s;
  size_t i = 0;
  size_t limit;
  std::string err;
  Parser(const std::string& str, size_t lim) : s(str), limit(lim) {}

  static int code(const std::string& n) {
    if (n == "RAAR") return ALGO_RAAR_H;
    if (n == "HIO") return ALGO_HIO_H;
    if (n == "ER") return ALGO_ER_H;
    if (n == "POSER") return ALGO_POSER_H;
    if (n == "POSHIO") return ALGO_POSHIO_H;
    if (n == "FHIO") return ALGO_FHIO_H;
    if (n == "KKT") return ALGO_KKT_H;
    if (n == "shrinkWrap") return ALGO_SHRINKWRAP_H;
    if (n == "TV") return ALGO_TV_H;
    if (n == "XCORRELATION") return ALGO_XCORRELATION_H;
    return -1;
  }
  bool expr(std::vector<int>& out) {
    bool first = true;
    for (;;) {
      if (!term(out, first)) return false;
      first = false;
      if (i < s.size() && s[i] == '+') { ++i; continue; }
      return true;
    }
  }
  bool term(std::vector<int>& out, bool first_term) {
    size_t st = i;
    long long n = 0;
    bool neg = false;
    if (i < s.size() && (s[i] == '+' || s[i] == '-')) { neg = s[i] == '-'; ++i; }
    size_t d0 = i;
    while (i < s.size() && isdigit((unsigned char)s[i])) { n = n * 10 + (s[i] - '0'); ++i; if (n > 1000000000LL) break; }
    if (i == d0) { err = "expected a count at '" + s.substr(st) + "'"; return false; }
    if (neg) n = -n;
    if (i >= s.size() || s[i] != '*') { err = "expected '*' after count at '" + s.substr(st) + "'"; return false; }
    ++i;
    if (n < 0 || (n == 0 && !first_term)) {
      err = "count " + std::to_string(n) + " at '" + s.substr(st) + "' never terminates in the reference parser";
      return false;
    }
    std::vector<int> body;
    if (i < s.size() && s[i] == '(') {
      ++i;
      if (!expr(body)) return false;
      if (i >= s.size() || s[i] != ')') { err = "missing ')'"; return false; }
      ++i;
    } else {
      size_t a = i;
      while (i < s.size() && s[i] != '+' && s[i] != ')' && s[i] != '(' && s[i] != '*') ++i;
      std::string name = s.substr(a, i - a);
      int c = code(name);
      if (c < 0) { err = "Algorithm " + name + " not found"; return false; }
      body.push_back(c);
    }
    for (long long k = 0; k < n; ++k) {
      if (out.size() + body.size() > limit) { err = "algorithm expands beyond the step limit"; return false; }
      out.insert(out.end(), body.begin(), body.end());
    }
    return true;
  }
};
}  // namespace

int algo_expand(const char* f, std::vector<int>& out, size_t limit) {
  if (!f) return set_error(CDX_ERR_ARG_H, "algorithm string is NULL");
  std::string s;
  for (const char* p = f; *p; ++p)
    if (*p != ' ' && *p != '\t' && *p != '\n' && *p != '\r') s.push_back(*p);
  if (s.empty()) return set_error(CDX_ERR_ALGO_H, "empty algorithm string");
  Parser P(s, limit);
  out.clear();
  if (!P.expr(out)) return set_error(CDX_ERR_ALGO_H, P.err);
  if (P.i != s.size()) return set_error(CDX_ERR_ALGO_H, "trailing characters at '" + s.substr(P.i) + "'");
  return 0;
}

// ------------------------------------------------------------------ .bin files
// struct imageFile {char type; int rows, cols, nchann, typesize;} (include/imageFile.hpp:11-17),
// 20 bytes with padding; type FLOAT = 3, FLOAT2 = 4 (imgio.c:223-243).
struct BinHeader {
  char type;
  char pad[3];
  int rows, cols, nchann, typesize;
};
static_assert(sizeof(BinHeader) == 20, "imageFile header is 20 bytes");

int read_bin(const char* path, int* rows, int* cols, int* is_complex, float* data, size_t cap) {
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(CDX_ERR_IO_H, std::string("cannot open ") + path);
  BinHeader h;
  if (fread(&h, sizeof h, 1, f) != 1) {
    fclose(f);
    return set_error(CDX_ERR_IO_H, std::string("file is empty: ") + path);
  }
  if (h.type != 3 && h.type != 4) {
    fclose(f);
    return set_error(CDX_ERR_IO_H, "FILETYPE unrecognized: " + std::to_string((int)h.type));
  }
  if (h.rows <= 0 || h.cols <= 0) {
    fclose(f);
    return set_error(CDX_ERR_IO_H, "bad image size in header");
  }
  *rows = h.rows;
  *cols = h.cols;
  *is_complex = h.type == 4;
  if (data) {
    size_t n = (size_t)h.rows * h.cols * (h.type == 4 ? 2 : 1);
    if (n > cap) {
      fclose(f);
      return set_error(CDX_ERR_ARG_H, "buffer too small for the image");
    }
    if (fread(data, sizeof(float), n, f) != n) {
      fclose(f);
      return set_error(CDX_ERR_IO_H, std::string("image data short: ") + path);
    }
  }
  fclose(f);
  return 0;
}

int write_bin(const char* path, const float* data, int rows, int cols, int is_complex) {
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(CDX_ERR_IO_H, std::string("cannot write ") + path);
  BinHeader h;
  memset(&h, 0, sizeof h);
  h.type = is_complex ? 4 : 3;
  h.rows = rows;
  h.cols = cols;
  h.nchann = 1;
  size_t n = (size_t)rows * cols * (is_complex ? 2 : 1);
  bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(data, sizeof(float), n, f) == n;
  fclose(f);
  return ok ? 0 : set_error(CDX_ERR_IO_H, std::string("short write: ") + path);
}

}  // namespace cdx
