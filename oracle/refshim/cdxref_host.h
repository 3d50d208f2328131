// Host emulation of the CUDA execution model for building the reference's
// hot-path sources as plain C++ (test infrastructure: the oracle pin).
// Kernels become host functions; a launch runs the body once per thread of
// the grid, with blockIdx/threadIdx/blockDim/gridDim as thread-local globals.
// Element-wise kernels run this way; kernels that synchronise their block
// (__syncthreads over extern shared memory) are launched through
// cdxref::coop, which runs each block's threads as OS threads, blocks in turn.
#pragma once
#include <algorithm>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>
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
// __syncthreads of a cooperative block: a generation-counted barrier; a thread
// that returns leaves the count
struct BlockBarrier {
  std::mutex m;
  std::condition_variable cv;
  int expected = 0, arrived = 0;
  long gen = 0;
  void wait() {
    std::unique_lock<std::mutex> l(m);
    const long g = gen;
    if (++arrived == expected) { arrived = 0; ++gen; cv.notify_all(); return; }
    cv.wait(l, [&] { return gen != g; });
  }
  void drop() {
    std::unique_lock<std::mutex> l(m);
    if (--expected > 0 && arrived == expected) { arrived = 0; ++gen; cv.notify_all(); }
  }
};
extern thread_local BlockBarrier* tl_block_barrier;
template <class F> struct Coop {
  dim3 g, b;
  F f;
  template <class... A> void operator()(A... a) const {
    const unsigned nt = b.x * b.y * b.z;
    for (unsigned bz = 0; bz < g.z; ++bz)
      for (unsigned by = 0; by < g.y; ++by)
        for (unsigned bx = 0; bx < g.x; ++bx) {
          BlockBarrier bar;
          bar.expected = (int)nt;
          std::vector<std::thread> th;
          th.reserve(nt);
          for (unsigned t = 0; t < nt; ++t)
            th.emplace_back([&, t] {
              gridDim = g;
              blockDim = b;
              blockIdx = {bx, by, bz};
              threadIdx = {t % b.x, (t / b.x) % b.y, t / (b.x * b.y)};
              tl_block_barrier = &bar;
              f(a...);
              tl_block_barrier = nullptr;
              bar.drop();
            });
          for (auto& x : th) x.join();
        }
  }
};
template <class F> Coop<F> coop(dim3 g, dim3 b, F f) { return {g, b, f}; }
template <class F> Coop<F> coop(dim3 g, dim3 b, size_t, F f) { return {g, b, f}; }
}  // namespace cdxref

inline void __syncthreads() {
  if (cdxref::tl_block_barrier) cdxref::tl_block_barrier->wait();
}
template <class A, class B> inline auto max(A a, B b) -> decltype(a + b) { return a > b ? a : b; }
template <class A, class B> inline auto min(A a, B b) -> decltype(a + b) { return a < b ? a : b; }
inline float __fdividef(float a, float b) { return a / b; }
inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
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
