// Host stand-in for curand: an xorshift stream per state.  Not bit-compatible
// with MRG32k3a; the oracle pin runs the restart path, which draws nothing.
#pragma once
#include "cdxref_host.h"
struct curandStateMRG32k3a { unsigned long long s; };
typedef curandStateMRG32k3a curandState;
inline void curand_init(unsigned long long seed, unsigned long long seq, unsigned long long, curandStateMRG32k3a* st) {
  st->s = (seed ^ (seq * 0x9e3779b97f4a7c15ULL)) | 1; }
inline unsigned long long cdxref_next(curandStateMRG32k3a* st) {
  st->s ^= st->s << 13; st->s ^= st->s >> 7; st->s ^= st->s << 17; return st->s; }
inline float curand_uniform(curandStateMRG32k3a* st) { return ((cdxref_next(st) >> 40) + 1) * (1.0f / 16777216.0f); }
inline float curand_normal(curandStateMRG32k3a* st) {
  float u1 = curand_uniform(st), u2 = curand_uniform(st);
  return std::sqrt(-2.f * std::log(u1)) * std::cos(6.2831853f * u2); }
inline unsigned int curand_poisson(curandStateMRG32k3a* st, double lambda) {
  if (lambda <= 0) return 0;
  if (lambda > 64) { double v = lambda + std::sqrt(lambda) * curand_normal(st); return v < 0 ? 0 : (unsigned)(v + 0.5); }
  double L = std::exp(-lambda), p = 1.0; unsigned k = 0;
  do { ++k; p *= curand_uniform(st); } while (p > L);
  return k - 1; }
