// Register-handoff Stockham engine and the FP32 iteration kernels built on it.
//
// Same transform and pass formula as fft_pass (cdx_fft.cuh), organised so
// that data enter and leave a CTA in registers:
//   * pass 0 loads its butterflies straight from global memory (no staging),
//   * the middle passes exchange through the skewed shared-memory lines,
//   * the last pass leaves its outputs in registers.
// A thread's last-pass outputs of plan 0 are element j + r*NS of line l for
// its butterflies (l, j); the first pass of plan 1 (the radices reversed)
// reads exactly those elements.  So the column pass runs
//     FFT (plan 0) -> projection in registers -> IFFT (plan 1) -> store,
// and the row pass
//     IFFT (plan 0) -> 1/N and update in registers -> FFT (plan 1) -> store,
// with two shared-memory exchanges per 2048-point transform and no staging of
// the lines in or out.
//
// Butterfly g of a pass (g = threadIdx.x + b*T) belongs to line
// l = (g >> cb) & (L-1) and index j = (g >> (cb + log2 L)) << cb | (g & (2^cb - 1)):
// with cb = 0 consecutive threads take consecutive lines (a column tile of
// width L is then read as one contiguous run); the row pass uses cb = log2 of
// the column tile width on tiled data, so 2^cb x L threads cover one piece of
// a tile, and the largest valid cb on row-major data.
// The map is the same for every pass of a kernel, which is what makes the
// register handoff valid.
#pragma once
#include "cdx_kernels.cuh"

namespace cdx {

template <int N, int PLAN, int P>
struct RPass {
  using G = Geom<N>;
  static constexpr int R = plan_radix_x(N, PLAN, P);
  static constexpr int NS = plan_ns_x(N, PLAN, P);
  static constexpr int NR = N / R;
  static constexpr int NB = G::L * NR;
  static constexpr int B = (NB + G::T - 1) / G::T;
  static constexpr int TWO = tw_offset_x(N, PLAN, P);
};

// Default butterfly chunk bits of the row pass on column-tiled data: the tile
// width (2^tl threads per tile row piece), except that 8-wide tiles take chunks
// of 16 where the length allows: with chunks of 8 a half-warp spans two lines
// whose stride is 2 mod 16 float2, so its shared-memory accesses conflict
// (512^2: 2.6 M bank conflicts per row pass), while 16 keep each half-warp on
// one line and still read whole 128-byte lines of W.
__host__ __device__ constexpr int row_cb_pick(int tl, int cb_max) {
  return tl == 3 && cb_max >= 4 ? 4 : (tl < cb_max ? tl : cb_max);
}

// largest chunk bits valid for every pass: NR = N / R is a multiple of 2^cb for
// every radix R of the length (both plans have the same radices), so the map
// below is a bijection onto (line, butterfly) in every pass; e.g. 2048 -> 7,
// 192 (NR 12, 48, 64) -> 2, 384 -> 3, 96 -> 1, 48 -> 0
template <int N>
__host__ __device__ constexpr int rfft_cb_max() {
  int c = 0;
  for (;;) {
    for (int p = 0; plan_radix(N, p) != 0; ++p)
      if ((N / plan_radix(N, p)) % (2 << c) != 0) return c;
    ++c;
  }
}

// (l, j) of butterfly b of this thread in a radix-R pass; false past the end
template <int N, int R>
__device__ __forceinline__ bool bfly_of(int b, int cb, int& l, int& j) {
  using G = Geom<N>;
  constexpr int NB = G::L * (N / R);
  const int g = threadIdx.x + b * G::T;
  if ((NB % G::T) != 0 && g >= NB) return false;
  l = (g >> cb) & (G::L - 1);
  j = ((g >> (cb + G::LOG2L)) << cb) | (g & ((1 << cb) - 1));
  return true;
}

// shared-memory word of element j + r*NR of line l (linear in r when NR % 16 == 0)
template <int N, int NR>
__device__ __forceinline__ int sidx_in(int l, int j, int r) {
  using G = Geom<N>;
  if constexpr (NR % 16 == 0) return G::idx(l, j) + r * (NR + NR / 16);
  else return G::idx(l, j + r * NR);
}
// shared-memory word of element base + r*NS of line l
template <int N, int R, int NS>
__device__ __forceinline__ int sidx_out(int l, int base, int r) {
  using G = Geom<N>;
  if constexpr (NS % 16 == 0) return G::idx(l, base) + r * (NS + NS / 16);
  else if constexpr (NS == 1 && R == 16) return G::idx(l, base) + r;   // base = 16 j
  else return G::idx(l, base + r * NS);
}

// twiddles and the radix-R DFT of one butterfly of pass P
template <int N, int PLAN, int P, bool INV>
__device__ __forceinline__ void rpass_compute(float2 (&v)[RPass<N, PLAN, P>::R], int j, const float2* tw) {
  using S = RPass<N, PLAN, P>;
  if constexpr (S::NS > 1) {
    const int k = j % S::NS;
#pragma unroll
    for (int r = 1; r < S::R; ++r) {
      float2 w = __ldg(tw + S::TWO + (r - 1) * S::NS + k);
      if (INV) w.y = -w.y;
      v[r] = cmul(v[r], w);
    }
  }
  dftR<S::R, INV>(v);
}

template <int N, int PLAN, int P>
__device__ __forceinline__ void rpass_store(float2* buf, float2 (&v)[RPass<N, PLAN, P>::B][RPass<N, PLAN, P>::R],
                                            int cb) {
  using S = RPass<N, PLAN, P>;
#pragma unroll
  for (int b = 0; b < S::B; ++b) {
    int l, j;
    if (!bfly_of<N, S::R>(b, cb, l, j)) continue;
    const int k = j % S::NS;
    const int base = (j - k) * S::R + k;
#pragma unroll
    for (int r = 0; r < S::R; ++r) buf[sidx_out<N, S::R, S::NS>(l, base, r)] = v[b][r];
  }
}

template <int N, int PLAN, int P>
__device__ __forceinline__ void rpass_load(const float2* buf, float2 (&v)[RPass<N, PLAN, P>::B][RPass<N, PLAN, P>::R],
                                           int cb) {
  using S = RPass<N, PLAN, P>;
#pragma unroll
  for (int b = 0; b < S::B; ++b) {
    int l, j;
    if (!bfly_of<N, S::R>(b, cb, l, j)) continue;
#pragma unroll
    for (int r = 0; r < S::R; ++r) v[b][r] = buf[sidx_in<N, S::NR>(l, j, r)];
  }
}

template <int N, int PLAN, int P, bool INV>
__device__ __forceinline__ void rpass_compute_all(float2 (&v)[RPass<N, PLAN, P>::B][RPass<N, PLAN, P>::R], int cb,
                                                  const float2* tw) {
  using S = RPass<N, PLAN, P>;
#pragma unroll
  for (int b = 0; b < S::B; ++b) {
    int l, j;
    if (!bfly_of<N, S::R>(b, cb, l, j)) continue;
    rpass_compute<N, PLAN, P, INV>(v[b], j, tw);
  }
}

// middle passes P .. M-2 through shared memory (each ends with a barrier)
template <int N, int PLAN, int P, bool INV>
__device__ __forceinline__ void rfft_middle(float2* buf, const float2* tw, int cb) {
  if constexpr (P < plan_len(N) - 1) {
    using S = RPass<N, PLAN, P>;
    float2 v[S::B][S::R];
    rpass_load<N, PLAN, P>(buf, v, cb);
    __syncthreads();
    rpass_compute_all<N, PLAN, P, INV>(v, cb, tw);
    rpass_store<N, PLAN, P>(buf, v, cb);
    __syncthreads();
    rfft_middle<N, PLAN, P + 1, INV>(buf, tw, cb);
  }
}

template <int N, int PLAN>
using RFirst = RPass<N, PLAN, 0>;
template <int N, int PLAN>
using RLast = RPass<N, PLAN, plan_len(N) - 1>;

struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// The whole transform of the CTA's L lines: `in` holds pass 0's inputs
// (element j + r*N/R0 of line l for butterfly (l, j)), `out` receives the
// last pass's outputs (element j + r*NS_last).  The shared lines must be free
// on entry (callers synchronise); on return other threads may still be
// reading them, so callers synchronise before the next write.  `hook` runs
// after every thread's last read of the shared lines has been issued and before
// the last pass's arithmetic (a caller that synchronises there may refill the
// lines while the last pass computes).
template <int N, int PLAN, bool INV, class H = NoHook>
__device__ __forceinline__ void rfft(float2 (&in)[RFirst<N, PLAN>::B][RFirst<N, PLAN>::R],
                                     float2 (&out)[RLast<N, PLAN>::B][RLast<N, PLAN>::R], float2* buf,
                                     const float2* tw, int cb, H&& hook = H{}) {
  constexpr int M = plan_len(N);
  rpass_compute_all<N, PLAN, 0, INV>(in, cb, tw);
  if constexpr (M == 1) {
#pragma unroll
    for (int b = 0; b < RFirst<N, PLAN>::B; ++b)
#pragma unroll
      for (int r = 0; r < RFirst<N, PLAN>::R; ++r) out[b][r] = in[b][r];
    hook();
  } else {
    rpass_store<N, PLAN, 0>(buf, in, cb);
    __syncthreads();
    rfft_middle<N, PLAN, 1, INV>(buf, tw, cb);
    rpass_load<N, PLAN, M - 1>(buf, out, cb);
    hook();
    rpass_compute_all<N, PLAN, M - 1, INV>(out, cb, tw);
  }
}

// Shared memory and resident CTAs per SM (register budget) of the
// register-handoff kernels.  The column pass at 256 threads is budgeted for 4
// CTAs per SM (64 registers, no spills; 2-4 % faster than 3).  The row pass
// stages its rho rows in the line buffer (loading rho straight from global
// memory instead was 4-30 % slower, its latency exposed) and is budgeted for 4
// CTAs per SM below 1024 and 3 from 1024 up, where the radix-16 last passes
// would spill at 64 registers (2048^2: 80 registers, 50.5 -> 49.7 us per
// iteration; 512^2 x16 is faster at 4).
#ifndef CDX_RK_MINB_COL
#define CDX_RK_MINB_COL 4
#endif

#ifndef CDX_RK_MINB_ROW
#define CDX_RK_MINB_ROW 0
#endif
// RHO_IN_BUF: the iterating row pass stages its rho rows in the FFT line buffer
// itself, copied in after the inverse transform's last shared-memory read (the
// copy overlaps the last pass's arithmetic), so the CTA needs one line buffer
// instead of two and four CTAs fit per SM instead of three.
#ifndef CDX_RHO_IN_BUF
#define CDX_RHO_IN_BUF 1
#endif
template <int N>
struct RGeom {
  using G = Geom<N>;
  static constexpr bool RHO_IN_BUF = CDX_RHO_IN_BUF && G::T == 256 && plan_len(N) > 1;
  static constexpr int SMEM_ROW_ITER =
      G::SMEM_LINES + (RHO_IN_BUF ? 0 : G::L * G::LD * (int)sizeof(float2)) + G::L * ((N + 31) >> 5) * 4;
  static constexpr int MINB_COL = (CDX_RK_MINB_COL > 0 && G::T == 256) ? CDX_RK_MINB_COL : G::MINB;
  static constexpr int MINB_ROW =
      (CDX_RK_MINB_ROW > 0 && G::T == 256) ? CDX_RK_MINB_ROW : (RHO_IN_BUF ? (N >= 1024 ? 3 : 4) : G::MINB);
};

// ------------------------------------------------------------- real-space updates
template <int ALGO>
__device__ __forceinline__ float2 update_t(bool inside, float2 x, float2 p, float beta) {
  return apply_update(ALGO, inside, x, p, beta);
}

// ---------------------------------------------------------------- column pass
// Lines are columns (length N = rows).  Column-tiled arrays have tile width L.
// PROJ (COL_ITER): the modulus projection, PROJ_MODABS or PROJ_CCD.
template <int N, int MODE, int PROJ>
__global__ void __launch_bounds__(Geom<N>::T, RGeom<N>::MINB_COL) col_pass_rk(ColArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  using F0 = RFirst<N, 0>;
  using FL = RLast<N, 0>;   // == RFirst<N, 1> in shape
  using IL = RLast<N, 1>;
  static_assert(FL::R == RFirst<N, 1>::R && FL::B == RFirst<N, 1>::B, "plan 1 starts where plan 0 ends");
  extern __shared__ float2 smem[];
  __shared__ double red[T / 32];
  pdl_wait_and_release();
  const float2* __restrict__ tw = a.tw;
  float2* buf = smem;
  const int c0 = blockIdx.x * L;
  const int ncols = min(L, a.cols - c0);
  const long long C = a.cols;
  const long long tile = (long long)blockIdx.x * N * L;

  if (a.state) {
    const int f = a.state[blockIdx.y].flags;
    if (f & 6) {
      if ((f & 4) == 0 && threadIdx.x == 0) atomicOr(&a.state[blockIdx.y].flags, 4);
      return;
    }
  }
  constexpr bool iter = MODE == COL_ITER;
  float* amp_s = reinterpret_cast<float*>(smem + L * G::LD);
  float* int_s = amp_s + L * N;
  float* bs_s = int_s + L * N;
  const long long aux = (long long)blockIdx.y * a.aux_stride + tile;
  // the tile's sqrt(I) (and I, beamstop for PROJ_CCD): contiguous runs of L*N
  // floats, one bulk copy each, landing during the forward transform
  __shared__ uint64_t stage_bar;
  if constexpr (iter) {
    if constexpr (bulk_staging<N>()) {
      constexpr unsigned bytes = L * N * (unsigned)sizeof(float);
      if (threadIdx.x == 0) bulk_bar_init(&stage_bar);
      __syncthreads();
      if (threadIdx.x == 0) {
        const bool two = PROJ == PROJ_CCD, three = PROJ == PROJ_CCD && a.bs != nullptr;
        bulk_expect(&stage_bar, bytes * (1u + (two ? 1u : 0u) + (three ? 1u : 0u)));
        bulk_g2s(amp_s, a.amp + aux, bytes, &stage_bar);
        if (two) bulk_g2s(int_s, a.inten + aux, bytes, &stage_bar);
        if (three) bulk_g2s(bs_s, a.bs + aux, bytes, &stage_bar);
      }
    } else {
#pragma unroll 4
      for (int q = threadIdx.x; q < L * N / 4; q += T) {
        cp_async16(amp_s + 4 * q, a.amp + aux + 4 * q, true);
        if constexpr (PROJ == PROJ_CCD) {
          cp_async16(int_s + 4 * q, a.inten + aux + 4 * q, true);
          if (a.bs) cp_async16(bs_s + 4 * q, a.bs + aux + 4 * q, true);
        }
      }
      cp_commit();
    }
  }
  const float2* in = a.in + (long long)blockIdx.y * a.in_stride;
  const bool in_t = a.in_tiled != 0;
  auto gload = [&](int l, int m) -> float2 {
    if (in_t) return __ldcg(in + tile + (long long)m * L + l);
    return l < ncols ? __ldcg(in + m * C + c0 + l) : make_float2(0.f, 0.f);
  };
  float2 v[FL::B][FL::R];
  const bool fwd_fft = !iter || !a.from_psi;
  if (fwd_fft) {
    float2 v0[F0::B][F0::R];
#pragma unroll
    for (int b = 0; b < F0::B; ++b) {
      int l, j;
      if (!bfly_of<N, F0::R>(b, 0, l, j)) continue;
#pragma unroll
      for (int r = 0; r < F0::R; ++r) v0[b][r] = gload(l, j + r * F0::NR);
    }
    if (!iter && a.inv) rfft<N, 0, true>(v0, v, buf, tw, 0);
    else rfft<N, 0, false>(v0, v, buf, tw, 0);
  } else {
    // Psi given: load it where the forward transform would have left it
#pragma unroll
    for (int b = 0; b < FL::B; ++b) {
      int l, j;
      if (!bfly_of<N, FL::R>(b, 0, l, j)) continue;
#pragma unroll
      for (int r = 0; r < FL::R; ++r) v[b][r] = gload(l, j + r * FL::NS);
    }
  }
  float2* out = a.out + (long long)blockIdx.y * a.out_stride;
  const bool out_t = a.out_tiled != 0;
  const float s = a.scale;
  if constexpr (!iter) {
#pragma unroll
    for (int b = 0; b < FL::B; ++b) {
      int l, j;
      if (!bfly_of<N, FL::R>(b, 0, l, j)) continue;
#pragma unroll
      for (int r = 0; r < FL::R; ++r) {
        const int m = j + r * FL::NS;
        float2 y = v[b][r];
        if (s != 1.f) { y.x *= s; y.y *= s; }
        if (out_t) __stcg(out + tile + (long long)m * L + l, y);
        else if (l < ncols) __stcg(out + m * C + c0 + l, y);
      }
    }
    return;
  } else {
    if constexpr (bulk_staging<N>()) bulk_wait(&stage_bar, a.err);
    else cp_wait<0>();
    __syncthreads();
    // Psi complete in registers: optional R-factor partial (one loop behind
    // one uniform branch), then the projection (branch-free per element, so
    // the compiler interleaves the elements), then the optional copy-out of P_M Psi
    if (a.rf_partials) {
      double rsum = 0.0;
#pragma unroll
      for (int b = 0; b < FL::B; ++b) {
        int l, j;
        if (!bfly_of<N, FL::R>(b, 0, l, j) || l >= ncols) continue;
#pragma unroll
        for (int r = 0; r < FL::R; ++r) {
          const float2 z = v[b][r];
          rsum += fabsf(hypotf(z.x, z.y) - amp_s[(j + r * FL::NS) * L + l]);
        }
      }
      const double tsum = block_sum_d<T>(rsum, red);
      if (threadIdx.x == 0) a.rf_partials[(long long)blockIdx.y * gridDim.x + blockIdx.x] = tsum;
    }
#pragma unroll
    for (int b = 0; b < FL::B; ++b) {
      int l, j;
      if (!bfly_of<N, FL::R>(b, 0, l, j)) continue;
#pragma unroll
      for (int r = 0; r < FL::R; ++r) {
        const int t = (j + r * FL::NS) * L + l;
        float2 z = v[b][r];
        if constexpr (PROJ == PROJ_MODABS) z = proj_modabs(z, amp_s[t]);
        else z = proj_ccd(z, int_s[t], a.bs ? bs_s[t] : 0.f, a.bs != nullptr, a.noise_level, a.ccd_scale,
                          a.ccd_rcolor);
        v[b][r] = l < ncols ? z : make_float2(0.f, 0.f);
      }
    }
    if (a.psi_out) {
      float2* psi_out = a.psi_out + (long long)blockIdx.y * a.psi_stride;
#pragma unroll
      for (int b = 0; b < FL::B; ++b) {
        int l, j;
        if (!bfly_of<N, FL::R>(b, 0, l, j) || l >= ncols) continue;
#pragma unroll
        for (int r = 0; r < FL::R; ++r) psi_out[(j + r * FL::NS) * C + c0 + l] = v[b][r];
      }
    }
    float2 o[IL::B][IL::R];
    rfft<N, 1, true>(v, o, buf, tw, 0);
#pragma unroll
    for (int b = 0; b < IL::B; ++b) {
      int l, j;
      if (!bfly_of<N, IL::R>(b, 0, l, j)) continue;
#pragma unroll
      for (int r = 0; r < IL::R; ++r) {
        const int m = j + r * IL::NS;
        float2 y = o[b][r];
        if (s != 1.f) { y.x *= s; y.y *= s; }
        if (out_t) __stcg(out + tile + (long long)m * L + l, y);
        else if (l < ncols) __stcg(out + m * C + c0 + l, y);
      }
    }
  }
}

// ------------------------------------------------------------------- row pass
// Lines are rows (length N = cols).  Column-tiled arrays have tile width
// 2^tile_log2 (the column pass's L for the row count).
// SQ (ROW_ITER only): W is column-tiled on both sides with the tile width of a
// column pass of length N (square patterns) and the butterflies use the default
// chunk, so the layout is known at compile time: each butterfly's 16 elements
// are one base address plus whole-tile strides, with no per-element index
// arithmetic.  The launcher takes the general kernel otherwise.
// The compile-time layout needs every pass's element stride to be whole tiles:
// 2^log2(L) divides N/R for each radix R (true from 256 up; at 16..192 the
// column tiles are wider than that).
template <int N>
__host__ __device__ constexpr bool row_sq_ok() { return Geom<N>::LOG2L <= rfft_cb_max<N>(); }

template <int N, int MODE, int ALGO, bool SQ = false>
__device__ __forceinline__ void row_pass_body(const RowArgs& a) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  using F0 = RFirst<N, 0>;
  using FL = RLast<N, 0>;
  using IL = RLast<N, 1>;
  static_assert(FL::R == RFirst<N, 1>::R && FL::B == RFirst<N, 1>::B, "plan 1 starts where plan 0 ends");
  extern __shared__ float2 smem[];
  const float2* __restrict__ tw = a.tw;
  float2* buf = smem;
  const int row0 = blockIdx.x * L;
  const int nrows = min(L, a.rows - row0);
  constexpr bool iter = MODE == ROW_ITER;
  constexpr bool CT = SQ && iter && row_sq_ok<N>();   // compile-time layout
  constexpr int TLC = G::LOG2L;
  constexpr int CBC = row_cb_pick(TLC, rfft_cb_max<N>());
  const int tl = CT ? TLC : a.tile_log2;
  // tiled: four (or 2^tl) threads per tile row piece; row-major: consecutive
  // threads take consecutive columns
  const bool tiled = a.in_tiled || a.out_tiled;
  const int cb = CT ? CBC
                    : (a.cb_plus1 > 0 ? min(a.cb_plus1 - 1, rfft_cb_max<N>())
                                      : (tiled ? row_cb_pick(tl, rfft_cb_max<N>()) : rfft_cb_max<N>()));

  // rho rows and support words of the CTA (ROW_ITER), landing during the inverse FFT
  // (RHO_IN_BUF: the rho rows land in the line buffer during its last pass)
  constexpr int RS = G::LD;                 // rho line stride in shared memory
  constexpr int WPR = (N + 31) >> 5;
  // Support words in shared memory: with MT the words a butterfly of the update
  // needs (columns j + r*NS, r < R: word (j >> 5) + r*NS/32) are staged next to
  // one another, so a thread reads its R words with R/4 16-byte loads instead of R.
  constexpr bool MT = FL::NS % 32 == 0 && FL::R % 4 == 0 && WPR % 4 == 0;
  constexpr int MG = MT ? FL::NS / 32 : 1;   // word groups per row
  auto mask_slot = [](int w) -> int {
    if constexpr (MT) {
      const int l = w / WPR, q = w - l * WPR;   // row l, word q = g + r*MG
      return l * WPR + (q % MG) * FL::R + q / MG;
    } else {
      return w;
    }
  };
  constexpr bool rho_in_buf = RGeom<N>::RHO_IN_BUF;
  float2* rho_s = rho_in_buf ? smem : smem + L * G::LD;
  uint32_t* mask_s = reinterpret_cast<uint32_t*>(smem + L * G::LD + (rho_in_buf ? 0 : L * RS));
  float2* rho = a.rho + (long long)blockIdx.y * a.rho_stride + (long long)row0 * N;
  // with an even line stride each rho row is one bulk copy (16-byte aligned)
  constexpr bool bulk_rho = bulk_staging<N>() && RS % 2 == 0;
  __shared__ uint64_t rho_bar;
  if constexpr (iter && bulk_rho) {
    if (threadIdx.x == 0) bulk_bar_init(&rho_bar);
    __syncthreads();
  }
  // the rho rows: one bulk copy per row, or 16- / 8-byte cp.async pieces
  auto stage_rho = [&]() {
    if constexpr (bulk_rho) {
      if (threadIdx.x == 0) {
        // the lines were last read through the generic proxy: order that before the bulk writes
        if constexpr (rho_in_buf) asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        bulk_expect(&rho_bar, (unsigned)nrows * N * (unsigned)sizeof(float2));
        for (int l = 0; l < nrows; ++l)
          bulk_g2s(rho_s + l * RS, rho + (long long)l * N, N * (unsigned)sizeof(float2), &rho_bar);
      }
    } else if constexpr (RS % 2 == 0) {
#pragma unroll 4
      for (int e = threadIdx.x; e < L * N / 2; e += T) {
        const int l = (2 * e) / N, c = 2 * e - l * N;
        const bool ok = l < nrows;
        cp_async16(rho_s + l * RS + c, ok ? rho + 2 * e : rho, ok);
      }
    } else {
#pragma unroll 4
      for (int e = threadIdx.x; e < L * N; e += T) {
        const int l = e / N, c = e - l * N;
        const bool ok = l < nrows;
        cp_async8(rho_s + l * RS + c, ok ? rho + e : rho, ok);
      }
    }
  };
  if constexpr (iter) {
    if constexpr (!rho_in_buf) stage_rho();
    // rows copied in late: start them towards L2 now
    if constexpr (rho_in_buf) if (threadIdx.x < nrows) bulk_prefetch_l2(rho + (long long)threadIdx.x * N, N * (unsigned)sizeof(float2));
    const uint32_t* mask = a.mask + (long long)blockIdx.y * a.mask_stride + (long long)row0 * WPR;
    for (int w = threadIdx.x; w < L * WPR; w += T) {
      const bool ok = w / WPR < nrows;
      cp_async4(mask_s + mask_slot(w), ok ? mask + w : mask, ok);
    }
    cp_commit();
  }
  const float2* in = a.in + (long long)blockIdx.y * a.in_stride;
  const long long R = a.rows;
  auto goff = [&](bool t, int l, int c) -> long long {
    const int row = row0 + l;
    return t ? ((((long long)(c >> tl)) * R + row) << tl) + (c & ((1 << tl) - 1)) : (long long)row * N + c;
  };
  float2 v[FL::B][FL::R];
  {
    float2 v0[F0::B][F0::R];
#pragma unroll
    for (int b = 0; b < F0::B; ++b) {
      int l, j;
      if (!bfly_of<N, F0::R>(b, cb, l, j)) continue;
      if constexpr (CT) {
        // element j + r*NR: tile (j >> TLC) + r*(NR >> TLC), lane j & (2^TLC - 1)
        static_assert(F0::NR % (1 << TLC) == 0, "first-pass stride is whole tiles");
        const float2* p = in + ((((long long)(j >> TLC)) * R + row0 + l) << TLC) + (j & ((1 << TLC) - 1));
        const long long st = ((long long)(F0::NR >> TLC) * R) << TLC;
#pragma unroll
        for (int r = 0; r < F0::R; ++r) v0[b][r] = l < nrows ? __ldcg(p + r * st) : make_float2(0.f, 0.f);
      } else {
#pragma unroll
        for (int r = 0; r < F0::R; ++r)
          v0[b][r] = l < nrows ? __ldcg(in + goff(a.in_tiled, l, j + r * F0::NR)) : make_float2(0.f, 0.f);
      }
    }
    if constexpr (iter && rho_in_buf) {
      rfft<N, 0, true>(v0, v, buf, tw, cb, [&]() {
        __syncthreads();   // every thread's last read of the lines is done
        stage_rho();
        cp_commit();
      });
    } else if (iter || a.inv) {
      rfft<N, 0, true>(v0, v, buf, tw, cb);
    } else {
      rfft<N, 0, false>(v0, v, buf, tw, cb);
    }
  }
  float2* out = a.out + (long long)blockIdx.y * a.out_stride;
  const float s = a.scale;
  if constexpr (!iter) {
#pragma unroll
    for (int b = 0; b < FL::B; ++b) {
      int l, j;
      if (!bfly_of<N, FL::R>(b, cb, l, j)) continue;
      if (l >= nrows) continue;
#pragma unroll
      for (int r = 0; r < FL::R; ++r) {
        float2 y = v[b][r];
        if (s != 1.f) { y.x *= s; y.y *= s; }
        __stcg(out + goff(a.out_tiled, l, j + r * FL::NS), y);
      }
    }
  } else {
    cp_wait<0>();
    if constexpr (bulk_rho) bulk_wait(&rho_bar, a.err);
    __syncthreads();
    // rho' = IFFT/N; update against rho and the support bits
#pragma unroll
    for (int b = 0; b < FL::B; ++b) {
      int l, j;
      if (!bfly_of<N, FL::R>(b, cb, l, j)) continue;
      const uint4* m4 = reinterpret_cast<const uint4*>(mask_s + l * WPR + (j >> 5) * FL::R);
      uint4 mq = make_uint4(0u, 0u, 0u, 0u);
#pragma unroll
      for (int r = 0; r < FL::R; ++r) {
        const int c = j + r * FL::NS;
        float2 y = make_float2(0.f, 0.f);
        if constexpr (MT) if ((r & 3) == 0) mq = m4[r >> 2];   // four words at a time
        if (l < nrows) {
          float2 p = v[b][r];
          p.x *= a.inv_n;
          p.y *= a.inv_n;
          const float2 x = rho_s[l * RS + c];
          const uint32_t word = MT ? ((r & 3) == 0 ? mq.x : (r & 3) == 1 ? mq.y : (r & 3) == 2 ? mq.z : mq.w)
                                   : mask_s[l * WPR + (c >> 5)];
          const bool inside = (word >> (c & 31)) & 1u;
          y = update_t<ALGO>(inside, x, p, a.beta);
          rho[l * N + c] = y;
        }
        v[b][r] = y;
      }
    }
    float2 o[IL::B][IL::R];
    if constexpr (rho_in_buf) __syncthreads();   // the rho rows are read before the lines are reused
    rfft<N, 1, false>(v, o, buf, tw, cb);
#pragma unroll
    for (int b = 0; b < IL::B; ++b) {
      int l, j;
      if (!bfly_of<N, IL::R>(b, cb, l, j)) continue;
      if (l >= nrows) continue;
      if constexpr (CT) {
        static_assert(IL::NS % (1 << TLC) == 0, "last-pass stride is whole tiles");
        float2* p = out + ((((long long)(j >> TLC)) * R + row0 + l) << TLC) + (j & ((1 << TLC) - 1));
        const long long st = ((long long)(IL::NS >> TLC) * R) << TLC;
#pragma unroll
        for (int r = 0; r < IL::R; ++r) __stcg(p + r * st, o[b][r]);   // the iteration stores unscaled
      } else {
#pragma unroll
        for (int r = 0; r < IL::R; ++r) {
          float2 y = o[b][r];
          if (s != 1.f) { y.x *= s; y.y *= s; }
          __stcg(out + goff(a.out_tiled, l, j + r * IL::NS), y);
        }
      }
    }
  }
}

// One kernel per update (ALGO is ignored in ROW_FFT mode): the executed code
// holds a single update and no switch.
template <int N, int MODE, int ALGO, bool SQ = false>
__global__ void __launch_bounds__(Geom<N>::T, RGeom<N>::MINB_ROW) row_pass_rk(RowArgs a) {
  pdl_wait_and_release();
  if (a.state && (a.state[blockIdx.y].flags & 4)) return;   // frozen pattern
  row_pass_body<N, MODE, ALGO, SQ>(a);
}
// the compile-time layout of row_pass_rk<..., true> applies to these arguments
template <int N>
__host__ __forceinline__ bool row_sq_layout(const RowArgs& a) {
  constexpr int cbd = row_cb_pick(Geom<N>::LOG2L, rfft_cb_max<N>());
  return row_sq_ok<N>() && a.mode == ROW_ITER && a.in_tiled && a.out_tiled && a.tile_log2 == Geom<N>::LOG2L && a.scale == 1.f &&
         (a.cb_plus1 == 0 || a.cb_plus1 - 1 == cbd);
}

}  // namespace cdx
