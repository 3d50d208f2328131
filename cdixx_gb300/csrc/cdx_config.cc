// readConfig and AlgoParser of the drop-in C++ layer (include/readConfig.hpp).
//
// The config files are libconfig text (the reference reads them with
// libconfig, src/independant/readConfig.cc:29-61).  This parser covers the
// subset the reference's configs use: `name = value;` / `name : value;`
// settings, `{ ... }` groups, `( ... )` lists and `[ ... ]` arrays (parsed and
// skipped), integers (decimal or hex, optional L), floats, booleans
// (true/false, any case), strings (adjacent literals concatenate, C escapes)
// and `#`, `//`, `/* */` comments.  Lookups follow the reference: ints from
// int settings (floats truncate, libconfig's auto-conversion), floats from
// float or int settings, bools from bool settings, strings from strings.
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

#include "../../include/readConfig.hpp"
#include "cdx_host.h"

namespace {

struct Val {
  enum Kind { INT, FLOAT, BOOL, STR, GROUP, OTHER } kind = OTHER;
  long long i = 0;
  double f = 0;
  bool b = false;
  std::string s;
};

struct CfgParser {
  std::string src;
  size_t p = 0;
  int line = 1;
  std::string err;
  std::map<std::string, Val> vals;

  void skip() {
    for (;;) {
      while (p < src.size() && isspace((unsigned char)src[p])) { if (src[p] == '\n') ++line; ++p; }
      if (p < src.size() && src[p] == '#') { while (p < src.size() && src[p] != '\n') ++p; continue; }
      if (p + 1 < src.size() && src[p] == '/' && src[p + 1] == '/') { while (p < src.size() && src[p] != '\n') ++p; continue; }
      if (p + 1 < src.size() && src[p] == '/' && src[p + 1] == '*') {
        p += 2;
        while (p + 1 < src.size() && !(src[p] == '*' && src[p + 1] == '/')) { if (src[p] == '\n') ++line; ++p; }
        p = std::min(src.size(), p + 2);
        continue;
      }
      return;
    }
  }
  bool fail(const std::string& m) {
    if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
    return false;
  }
  bool name(std::string& out) {
    skip();
    size_t a = p;
    if (p < src.size() && (isalpha((unsigned char)src[p]) || src[p] == '*')) {
      ++p;
      while (p < src.size() && (isalnum((unsigned char)src[p]) || src[p] == '_' || src[p] == '*' || src[p] == '-')) ++p;
    }
    if (p == a) return fail("setting name expected");
    out = src.substr(a, p - a);
    return true;
  }
  bool string_lit(std::string& out) {
    out.clear();
    for (;;) {
      skip();
      if (p >= src.size() || src[p] != '"') return true;
      ++p;
      while (p < src.size() && src[p] != '"') {
        char c = src[p++];
        if (c == '\\' && p < src.size()) {
          char e = src[p++];
          c = e == 'n' ? '\n' : e == 't' ? '\t' : e == 'r' ? '\r' : e == 'f' ? '\f' : e;
        }
        if (c == '\n') ++line;
        out.push_back(c);
      }
      if (p >= src.size()) return fail("unterminated string");
      ++p;
    }
  }
  bool value(const std::string& path, Val& v) {
    skip();
    if (p >= src.size()) return fail("value expected");
    char c = src[p];
    if (c == '{') {
      ++p;
      v.kind = Val::GROUP;
      return settings(path + ".", '}');
    }
    if (c == '(' || c == '[') {
      const char close = c == '(' ? ')' : ']';
      ++p;
      v.kind = Val::OTHER;
      int k = 0;
      for (;;) {
        skip();
        if (p < src.size() && src[p] == close) { ++p; return true; }
        Val sub;
        if (!value(path + "[" + std::to_string(k++) + "]", sub)) return false;
        skip();
        if (p < src.size() && src[p] == ',') ++p;
      }
    }
    if (c == '"') {
      v.kind = Val::STR;
      return string_lit(v.s);
    }
    size_t a = p;
    while (p < src.size() && (isalnum((unsigned char)src[p]) || strchr("+-._", src[p]))) ++p;
    std::string t = src.substr(a, p - a);
    if (t.empty()) return fail("value expected");
    std::string lt;
    for (char ch : t) lt.push_back((char)tolower((unsigned char)ch));
    if (lt == "true" || lt == "false") {
      v.kind = Val::BOOL;
      v.b = lt == "true";
      return true;
    }
    const bool hex = lt.size() > 2 && (lt.compare(0, 2, "0x") == 0 || lt.compare(0, 3, "-0x") == 0);
    const bool isfloat = !hex && (lt.find('.') != std::string::npos || lt.find('e') != std::string::npos);
    char* end = nullptr;
    if (isfloat) {
      v.kind = Val::FLOAT;
      v.f = strtod(t.c_str(), &end);
    } else {
      v.kind = Val::INT;
      v.i = strtoll(t.c_str(), &end, hex ? 16 : 10);
      if (end && (*end == 'L' || *end == 'l')) ++end;
      if (end && (*end == 'L' || *end == 'l')) ++end;
    }
    if (!end || *end != '\0') return fail("malformed value '" + t + "'");
    return true;
  }
  bool settings(const std::string& prefix, char close) {
    for (;;) {
      skip();
      if (p >= src.size()) return close == 0 ? true : fail("unexpected end of file");
      if (close && src[p] == close) {
        ++p;
        skip();
        if (p < src.size() && (src[p] == ';' || src[p] == ',')) ++p;
        return true;
      }
      std::string n;
      if (!name(n)) return false;
      skip();
      if (p >= src.size() || (src[p] != '=' && src[p] != ':')) return fail("'=' or ':' expected after " + n);
      ++p;
      Val v;
      if (!value(prefix + n, v)) return false;
      if (v.kind != Val::GROUP) {
        skip();
        if (p < src.size() && (src[p] == ';' || src[p] == ',')) ++p;
      }
      vals[prefix + n] = v;
    }
  }
};

}  // namespace

readConfig::readConfig(const char* configfile) {
  FILE* f = configfile ? fopen(configfile, "rb") : nullptr;
  if (!f) {
    fprintf(stderr, "%s:0 - file I/O error\n", configfile ? configfile : "(null)");
    exit(EXIT_FAILURE);
  }
  CfgParser P;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) P.src.append(buf, n);
  fclose(f);
  if (!P.settings("", 0)) {
    fprintf(stderr, "%s:%s\n", configfile, P.err.c_str());
    exit(EXIT_FAILURE);
  }
  printf("config file: %s\n", configfile);
  auto str = [&](const std::string& key, const char*& dst) {
    auto it = P.vals.find(key);
    if (it == P.vals.end() || it->second.kind != Val::STR) return;
    strings_.emplace_back(new std::string(it->second.s));
    dst = strings_.back()->c_str();
  };
  auto gint = [&](const char* k, int& dst) {
    auto it = P.vals.find(std::string("Job.") + k);
    if (it == P.vals.end()) return;
    if (it->second.kind == Val::INT) dst = (int)it->second.i;
    else if (it->second.kind == Val::FLOAT) dst = (int)it->second.f;
  };
  auto gll = [&](const char* k, long long& dst) {
    auto it = P.vals.find(std::string("Job.") + k);
    if (it != P.vals.end() && it->second.kind == Val::INT) dst = it->second.i;
  };
  auto gbool = [&](const char* k, bool& dst) {
    auto it = P.vals.find(std::string("Job.") + k);
    if (it != P.vals.end() && it->second.kind == Val::BOOL) dst = it->second.b;
  };
  auto gfloat = [&](const char* k, double& dst) {
    auto it = P.vals.find(std::string("Job.") + k);
    if (it == P.vals.end()) return;
    if (it->second.kind == Val::FLOAT) dst = it->second.f;
    else if (it->second.kind == Val::INT) dst = (double)it->second.i;
  };
  auto gstr = [&](const char* k, const char*& dst) { str(std::string("Job.") + k, dst); };
  for (const char* g : {"default", "pupil"}) {
    CDIfiles& fl = std::string(g) == "default" ? common : pupil;
    const std::string b = std::string("InputImages.") + g + ".";
    str(b + "Intensity", fl.Intensity);
    str(b + "Phase", fl.Phase);
    str(b + "restart", fl.restart);
    str(b + "Pattern", fl.Pattern);
  }
#define CDX_I(x) gint(#x, x);
#define CDX_B(x) gbool(#x, x);
#define CDX_F(x) gfloat(#x, x);
#define CDX_S(x) gstr(#x, x);
  CDX_I(beamStopSize) CDX_I(nIter) CDX_I(nIterpupil) CDX_I(noiseLevel) CDX_I(noiseLevel_pupil) CDX_I(verbose)
  CDX_I(mnistN) CDX_I(cropPattern) CDX_I(spectrumSamplingStep) CDX_I(saveVideoEveryIter) CDX_I(prtfIter)
  CDX_I(zernikeIter) CDX_I(scanx) CDX_I(scany) CDX_I(computeErrorEveryIter)
  CDX_B(isFlip) CDX_B(runSim) CDX_B(simCCDbit) CDX_B(isFresnel) CDX_B(doIteration) CDX_B(useGaussionLumination)
  CDX_B(useGaussionHERALDO) CDX_B(doCentral) CDX_B(useRectHERALDO) CDX_B(dopupil) CDX_B(useDM) CDX_B(useBS)
  CDX_B(reconAC) CDX_B(phaseModulation_pupil) CDX_B(intensityModulation) CDX_B(restart) CDX_B(saveIter)
  CDX_B(domnist) CDX_B(saveLMDB) CDX_B(solveSpectrum) CDX_B(mPIE) CDX_B(online)
  CDX_F(exposure) CDX_F(exposurepupil) CDX_F(oversampling) CDX_F(oversampling_spt) CDX_F(lambda) CDX_F(d)
  CDX_F(dpupil) CDX_F(pixelsize) CDX_F(beamspotsize) CDX_F(shrinkThreshold) CDX_F(positionUncertainty)
  CDX_F(costheta) CDX_F(photoncount) CDX_F(phaseModulation) CDX_F(stepSize) CDX_F(pupilSize)
  CDX_S(mnistData) CDX_S(algorithm) CDX_S(ccd_response) CDX_S(spectrum) CDX_S(BSimage) CDX_S(outputDir)
  CDX_S(distFile)
  CDX_F(beta) CDX_I(shrinkMode) CDX_F(sigma0) CDX_F(sigmaMin) CDX_F(sigmaDecay)
#undef CDX_I
#undef CDX_B
#undef CDX_F
#undef CDX_S
  gll("seed", seed);
}

void readConfig::print() {
  auto s = [](const char* x) { return x ? x : "(null)"; };
  printf("common Intensity=%s\ncommon Phase=%s\ncommon restart=%s\ncommon Pattern=%s\n", s(common.Intensity),
         s(common.Phase), s(common.restart), s(common.Pattern));
  printf("pupil Intensity=%s\npupil Phase=%s\npupil restart=%s\npupil Pattern=%s\n", s(pupil.Intensity),
         s(pupil.Phase), s(pupil.restart), s(pupil.Pattern));
  printf("algorithm = %s\nshrinkThreshold = %g\noversampling_spt = %g\nexposure = %g\nbeta = %g\n", s(algorithm),
         shrinkThreshold, oversampling_spt, exposure, beta);
}

AlgoParser::AlgoParser(const char* formula) {
  if (cdx::algo_expand(formula, steps_, 50000000)) {
    printf("%s\n", cdx::last_error());   // the reference prints "Algorithm X not found" and exits
    exit(0);
  }
  pos_ = 0;
}

void AlgoParser::restart() { pos_ = 0; }

int AlgoParser::next() { return pos_ < steps_.size() ? steps_[pos_++] : -1; }
