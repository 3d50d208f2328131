// Host stand-in for cub::DeviceReduce (used by the reference's cub_wrap.cu):
// a left-to-right fold with the given operator.
#pragma once
#include "../cuda_runtime.h"
namespace cub {
template <class K, class V> struct KeyValuePair { K key; V value; };
struct DeviceReduce {
  template <class In, class Out, class Op, class T>
  static int Reduce(void* tmp, size_t& bytes, In in, Out out, long long n, Op op, T init) {
    if (!tmp) { bytes = 16; return 0; }
    T acc = init;
    for (long long i = 0; i < n; ++i) acc = op(acc, in[i]);
    *out = acc;
    return 0;
  }
  template <class In, class V, class K>
  static int ArgMax(void* tmp, size_t& bytes, In in, V* vout, K* kout, long long n) {
    if (!tmp) { bytes = 16; return 0; }
    long long b = 0;
    for (long long i = 1; i < n; ++i) if (in[i] > in[b]) b = i;
    *vout = in[b]; *kout = (K)b;
    return 0;
  }
};
}  // namespace cub
