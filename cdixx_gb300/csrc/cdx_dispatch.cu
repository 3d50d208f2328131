// Length -> kernel dispatch for the row/column passes, and the twiddle tables.
#include <algorithm>
#include <atomic>
#include <cmath>

#include "cdx_fft.cuh"
#include "cdx_rfft.cuh"
#include "cdx_types.h"

namespace cdx {

template <int N> cudaError_t prepare_len();
template <int N> cudaError_t launch_row(const RowArgs&, int, cudaStream_t);
template <int N> cudaError_t launch_col(const ColArgs&, int, cudaStream_t);

#define CDX_FOR_EACH_SIZE(X) \
  X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) \
  X(1536) X(2048) X(3072) X(4096)

#define CASE_PREP(N) case N: return &prepare_len<N>;
#define CASE_ROW(N) case N: return &launch_row<N>;
#define CASE_COL(N) case N: return &launch_col<N>;
#define CASE_L(N) case N: return Geom<N>::L;
#define CASE_TW(N) case N: return Geom<N>::TWN;

PrepLaunch prep_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_PREP) default: return nullptr; }
}
RowLaunch row_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_ROW) default: return nullptr; }
}
ColLaunch col_launcher(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_COL) default: return nullptr; }
}
int lines_per_cta(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_L) default: return 0; }
}
int twiddle_count(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_TW) default: return 0; }
}
#define CASE_CB(N) case N: return rfft_cb_max<N>();
int row_cb_max(int n) {
  switch (n) { CDX_FOR_EACH_SIZE(CASE_CB) default: return 0; }
}
int row_cb_default(int n, int tile_log2) { return row_cb_pick(tile_log2, row_cb_max(n)); }

// Entry (r-1)*NS + k of pass p's block = W_n^(r*k*n/(NS*R)), W_n = exp(-2 pi i/n),
// evaluated in double with the exponent reduced mod n and rounded once to float;
// both radix plans of the length.
void twiddle_table(int n, float2* out) {
  const double two_pi = 6.283185307179586476925286766559;
  for (int plan = 0; plan < 2; ++plan)
    for (int p = 1; plan_radix_x(n, plan, p) != 0; ++p) {
      const int R = plan_radix_x(n, plan, p), NS = plan_ns_x(n, plan, p), step = n / (NS * R);
      float2* blk = out + tw_offset_x(n, plan, p);
      for (int r = 1; r < R; ++r)
        for (int k = 0; k < NS; ++k) {
          const long long t = ((long long)r * k * step) % n;
          const double a = two_pi * (double)t / (double)n;
          blk[(r - 1) * NS + k] = make_float2((float)std::cos(a), (float)-std::sin(a));
        }
    }
}

int sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
  if (dev < 64) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) return 1;
  if (dev < 64) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

}  // namespace cdx
