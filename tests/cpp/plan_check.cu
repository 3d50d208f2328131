// Host checks of the FFT plans and twiddle-table layout of cdx_fft.cuh and of
// the row pass's butterfly chunk bound (cdx_rfft.cuh), for every supported
// length: prints one line per length and "plans ok" when every check holds.
#include <cstdio>
#include <algorithm>
#include <vector>

#include "cdx_rfft.cuh"

using namespace cdx;

template <int N>
bool check_len() {
  bool ok = true;
  auto fail = [&](const char* what) {
    std::printf("N=%d: %s\n", N, what);
    ok = false;
  };
  const int m = plan_len(N);
  // radices multiply to N; the multiset is the largest-first one; plan 1 reverses plan 0
  long long prod = 1;
  std::vector<int> a, b;
  for (int p = 0; p < m; ++p) {
    prod *= plan_radix(N, p);
    a.push_back(plan_radix(N, p));
    b.push_back(radix_desc(N, p));
    if (plan_radix_x(N, 1, p) != plan_radix(N, m - 1 - p)) fail("plan 1 is not plan 0 reversed");
  }
  if (prod != N) fail("radices do not multiply to N");
  std::vector<int> sa = a, sb = b;
  std::sort(sa.begin(), sa.end());
  std::sort(sb.begin(), sb.end());
  if (sa != sb) fail("plan radices differ from the length's radices");
  // V: the first two radices of radix_desc (the largest-first order) sit at the two ends
  if (m >= 2 && !((a[0] == b[0] && a[m - 1] == b[1]) || (a[0] == b[1] && a[m - 1] == b[0])))
    fail("the ends are not the two leading radices");
  // twiddle blocks: (R-1)*NS entries per pass, inside the table, disjoint within a plan;
  // a plan that reads the same both ways uses plan 0's blocks for plan 1
  const bool same = plans_same(N);
  for (int plan = 0; plan < 2; ++plan) {
    int expect = (plan == 0 || same) ? 0 : tw_plan_count(N, 0);
    for (int p = 1; p < m; ++p) {
      if (tw_offset_x(N, plan, p) != expect) fail("twiddle block offset");
      expect += (plan_radix_x(N, plan, p) - 1) * plan_ns_x(N, plan, p);
      if (expect > tw_count(N)) fail("twiddle block past the table");
      if (same && tw_offset_x(N, 1, p) != tw_offset_x(N, 0, p)) fail("symmetric plan does not share blocks");
    }
  }
  // chunk bound: 2^cb divides N/R for every radix; the compile-time row layout only where valid
  const int cb = rfft_cb_max<N>();
  for (int p = 0; p < m; ++p)
    if ((N / plan_radix(N, p)) % (1 << cb) != 0) fail("chunk bits too large");
  if (row_sq_ok<N>() != (Geom<N>::LOG2L <= cb)) fail("row_sq_ok");
  // the butterfly -> (line, index) map of a pass is a bijection for every chunk width the
  // row pass may take (the tuner's variants and the default of any tile width)
  for (int c = 0; c <= cb; ++c)
    for (int p = 0; p < m; ++p) {
      const int R = plan_radix(N, p), L = Geom<N>::L, NR = N / R, NB = L * NR;
      std::vector<char> seen(NB, 0);
      for (int g = 0; g < NB; ++g) {
        const int l = (g >> c) & (L - 1);
        const int j = ((g >> (c + Geom<N>::LOG2L)) << c) | (g & ((1 << c) - 1));
        if (l >= L || j >= NR || seen[l * NR + j]++) { fail("butterfly map is not a bijection"); break; }
      }
    }
  for (int tl = 0; tl <= 8; ++tl)
    if (row_cb_pick(tl, cb) > cb || row_cb_pick(tl, cb) < 0) fail("default chunk past the bound");
  std::printf("N=%d plan", N);
  for (int r : a) std::printf(" %d", r);
  std::printf(" twiddles %d%s cb_max %d sq %d\n", tw_count(N), same ? " (shared)" : "", cb, (int)row_sq_ok<N>());
  return ok;
}

int main() {
  bool ok = check_len<16>() & check_len<24>() & check_len<32>() & check_len<48>() & check_len<64>() &
            check_len<96>() & check_len<128>() & check_len<192>() & check_len<256>() & check_len<384>() &
            check_len<512>() & check_len<768>() & check_len<1024>() & check_len<1536>() & check_len<2048>() &
            check_len<3072>() & check_len<4096>();
  std::printf(ok ? "plans ok\n" : "plans FAILED\n");
  return ok ? 0 : 1;
}
