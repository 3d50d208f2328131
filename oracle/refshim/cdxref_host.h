// Host emulation of the CUDA execution model for building the reference's
// hot-path sources as plain C++ (test infrastructure: the oracle pin).
// Kernels become host functions; a launch runs the body once per thread of
// the grid, with blockIdx/threadIdx/blockDim/gridDim as thread-local globals.
// Only element-wise kernels (no __syncthreads) are ever executed this way.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __constant__
#define __shared__
#define __restrict__
#define __align__(n)
#define __noinline__

struct dim3 {
  unsigned x = 1, y = 1, z = 1;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3_t { unsigned x, y, z; };
extern thread_local uint3_t blockIdx, threadIdx;
extern thread_local dim3 blockDim, gridDim;

namespace cdxref {
struct Launch {
  dim3 g, b;
  long long i = -1, n;
  Launch(dim3 grid, dim3 block, size_t = 0, void* = nullptr) : g(grid), b(block) {
    n = (long long)g.x * g.y * g.z * b.x * b.y * b.z;
    gridDim = g;
    blockDim = b;
  }
  bool next() {
    if (++i >= n) return false;
    long long t = i;
    threadIdx.x = t % b.x; t /= b.x;
    threadIdx.y = t % b.y; t /= b.y;
    threadIdx.z = t % b.z; t /= b.z;
    blockIdx.x = t % g.x; t /= g.x;
    blockIdx.y = t % g.y; t /= g.y;
    blockIdx.z = (unsigned)t;
    return true;
  }
};
}  // namespace cdxref

inline void __syncthreads() {}
template <class A, class B> inline auto max(A a, B b) -> decltype(a + b) { return a > b ? a : b; }
template <class A, class B> inline auto min(A a, B b) -> decltype(a + b) { return a < b ? a : b; }
inline float __fdividef(float a, float b) { return a / b; }
inline float __expf(float a) { return std::exp(a); }
inline float __logf(float a) { return std::log(a); }
inline float __sinf(float a) { return std::sin(a); }
inline float __cosf(float a) { return std::cos(a); }
inline float __saturatef(float a) { return a < 0 ? 0 : (a > 1 ? 1 : a); }
inline float rsqrtf(float a) { return 1.f / std::sqrt(a); }
inline int __float2int_rn(float a) { return (int)std::nearbyint(a); }
inline float atomicAdd(float* p, float v) { float o = *p; *p += v; return o; }
inline double atomicAdd(double* p, double v) { double o = *p; *p += v; return o; }
inline int atomicAdd(int* p, int v) { int o = *p; *p += v; return o; }
inline unsigned atomicAdd(unsigned* p, unsigned v) { unsigned o = *p; *p += v; return o; }
using std::exp; using std::sqrt; using std::log; using std::sin; using std::cos; using std::atan2; using std::floor;
using std::ceil; using std::fabs; using std::pow; using std::hypot; using std::abs; using std::round;
inline unsigned __float_as_uint(float f) { unsigned u; memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned u) { float f; memcpy(&f, &u, 4); return f; }
inline int __float_as_int(float f) { int u; memcpy(&u, &f, 4); return u; }
inline float __int_as_float(int u) { float f; memcpy(&f, &u, 4); return f; }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __clz(int x) { return x ? __builtin_clz((unsigned)x) : 32; }
inline double rsqrt(double a) { return 1.0 / std::sqrt(a); }
inline float exp10f(float a) { return std::pow(10.f, a); }
inline float sinpif(float a) { return std::sin((float)M_PI * a); }
inline float cospif(float a) { return std::cos((float)M_PI * a); }
inline void sincospif(float a, float* s, float* c) { *s = sinpif(a); *c = cospif(a); }
