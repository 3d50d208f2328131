// Host stand-in for the cuFFT C2C (and R2C) plans the reference uses (cudaConfig.cu:137-180):
// the published unnormalised DFT, evaluated in double (radix-2 for powers of
// two, direct sums otherwise) and rounded once to float.
#pragma once
#include <complex>
#include <map>
#include <vector>
#include "cuda_runtime.h"
typedef int cufftHandle;
typedef int cufftResult;
typedef float2 cufftComplex;
typedef float cufftReal;
enum { CUFFT_SUCCESS = 0 };
enum cufftType { CUFFT_C2C = 0x29, CUFFT_R2C = 0x2a, CUFFT_C2R = 0x2c };
enum { CUFFT_FORWARD = -1, CUFFT_INVERSE = 1 };
struct cdxref_plan { int rows, cols, batch; };
std::map<int, cdxref_plan>& cdxref_plans();
inline cufftResult cufftPlan2d(cufftHandle* h, int nx, int ny, int) {
  static int next = 1; *h = next++; cdxref_plans()[*h] = {nx, ny, 1}; return 0; }
inline cufftResult cufftPlan1d(cufftHandle* h, int n, int, int batch) {
  static int next = 100000; *h = next++; cdxref_plans()[*h] = {n, 1, batch}; return 0; }
inline cufftResult cufftPlanMany(cufftHandle* h, int, int* n, int*, int, int, int*, int, int, int, int batch) {
  return cufftPlan1d(h, n[0], 0, batch); }
inline cufftResult cufftDestroy(cufftHandle) { return 0; }
inline void cdxref_dft1(std::vector<std::complex<double>>& a, int dir) {
  const size_t n = a.size();
  if (n <= 1) return;
  if ((n & (n - 1)) == 0) {
    for (size_t i = 1, j = 0; i < n; ++i) {
      size_t bit = n >> 1;
      for (; j & bit; bit >>= 1) j ^= bit;
      j ^= bit;
      if (i < j) std::swap(a[i], a[j]);
    }
    for (size_t len = 2; len <= n; len <<= 1) {
      for (size_t i = 0; i < n; i += len)
        for (size_t k = 0; k < len / 2; ++k) {
          const double ang = dir * 2.0 * M_PI * (double)k / (double)len;
          const std::complex<double> w(std::cos(ang), std::sin(ang));
          std::complex<double> u = a[i + k], v = a[i + k + len / 2] * w;
          a[i + k] = u + v;
          a[i + k + len / 2] = u - v;
        }
    }
    return;
  }
  std::vector<std::complex<double>> out(n);
  for (size_t k = 0; k < n; ++k) {
    std::complex<double> s = 0;
    for (size_t t = 0; t < n; ++t) {
      const double ang = dir * 2.0 * M_PI * (double)((k * t) % n) / (double)n;
      s += a[t] * std::complex<double>(std::cos(ang), std::sin(ang));
    }
    out[k] = s;
  }
  a.swap(out);
}
inline cufftResult cufftExecC2C(cufftHandle h, cufftComplex* in, cufftComplex* out, int dir) {
  const cdxref_plan p = cdxref_plans().at(h);
  const int R = p.rows, C = p.cols;
  std::vector<std::complex<double>> a((size_t)R * C), line;
  for (size_t i = 0; i < a.size(); ++i) a[i] = {in[i].x, in[i].y};
  line.resize(C);
  for (int r = 0; r < R; ++r) {
    for (int c = 0; c < C; ++c) line[c] = a[(size_t)r * C + c];
    cdxref_dft1(line, dir);
    for (int c = 0; c < C; ++c) a[(size_t)r * C + c] = line[c];
  }
  if (C > 1) {
    line.resize(R);
    for (int c = 0; c < C; ++c) {
      for (int r = 0; r < R; ++r) line[r] = a[(size_t)r * C + c];
      cdxref_dft1(line, dir);
      for (int r = 0; r < R; ++r) a[(size_t)r * C + c] = line[r];
    }
  }
  for (size_t i = 0; i < a.size(); ++i) out[i] = {(float)a[i].real(), (float)a[i].imag()};
  return 0;
}
// R2C: the C2C transform of the real input, columns 0 .. cols/2 of each row kept
inline cufftResult cufftExecR2C(cufftHandle h, cufftReal* in, cufftComplex* out) {
  const cdxref_plan p = cdxref_plans().at(h);
  const int R = p.rows, C = p.cols, H = C / 2 + 1;
  std::vector<cufftComplex> full((size_t)R * C);
  for (size_t i = 0; i < full.size(); ++i) full[i] = {in[i], 0.f};
  cufftExecC2C(h, full.data(), full.data(), CUFFT_FORWARD);
  for (int r = 0; r < R; ++r)
    for (int c = 0; c < H; ++c) out[(size_t)r * H + c] = full[(size_t)r * C + c];
  return 0;
}
inline cufftResult cufftExecC2R(cufftHandle, cufftComplex*, cufftReal*) { abort(); }
