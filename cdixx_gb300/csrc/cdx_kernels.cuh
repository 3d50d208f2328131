// Fused CDI iteration kernels (sm_103a).
//
// One CDI iteration of the reference (src/post_gpu/cdi.cc:349-381) is
//     Psi <- P_M(Psi)                     applyModAbs / applyMod
//     rho' <- IFFT2(Psi) / (rows*cols)    myIFFT + applyNorm
//     rho  <- U(rho, rho', support)       Apply{HIO,RAAR,ER,...}Support
//     Psi  <- FFT2(rho)                   myFFT
// Here it is two kernels over a work buffer W that holds X = rowFFT(rho)
// between iterations:
//   column pass (one CTA = L whole columns):  colFFT(X) = Psi -> P_M -> colIFFT -> W
//   row pass    (one CTA = L whole rows):     rowIFFT(W)/N = rho' -> U -> rho,
//                                             rowFFT(rho) -> W
// so every pixel crosses HBM a fixed number of times per iteration and the
// projections never see their own launch.
#pragma once
#include "cdx_fft.cuh"
#include "cdx_types.h"

namespace cdx {

// ------------------------------------------------------------------ updates
// Real-space updates of src/gpu/cdi.cu:518-616, dispatched like applySupport
// (src/post_gpu/cdi.cc:25-36): unknown codes take the FHIO branch.  The
// reference forms x + 1.9*(p - x) and x - 1.2*p in double (double literals);
// here 1.9 and 1.2 are split into a float head and tail so two FMAs give the
// double-literal product to well below float resolution of the result.
__device__ __forceinline__ float relax19(float x, float p) {
  const float hi = 1.89999997615814209f;        // (float)1.9
  const float lo = 2.3841857821338408e-08f;     // 1.9 - (float)1.9
  float d = p - x;
  return fmaf(hi, d, fmaf(lo, d, x));
}
__device__ __forceinline__ float minus12(float x, float p) {
  const float hi = 1.20000004768371582f;        // (float)1.2
  const float lo = -4.7683715865426467e-08f;    // 1.2 - (float)1.2
  return fmaf(-hi, p, fmaf(-lo, p, x));
}

__device__ __forceinline__ float2 apply_update(int algo, bool inside, float2 x, float2 p, float beta) {
  switch (algo) {
    case ALGO_HIO:
      return inside ? p : make_float2(x.x - beta * p.x, x.y - beta * p.y);
    case ALGO_RAAR: {
      const float c = 1.f - 2.f * beta;
      return inside ? p : make_float2(beta * x.x + c * p.x, beta * x.y + c * p.y);
    }
    case ALGO_ER:
      return inside ? make_float2(relax19(x.x, p.x), relax19(x.y, p.y)) : make_float2(0.f, 0.f);
    case ALGO_POSER:
      return (inside && p.x > 0.f) ? p : make_float2(0.f, 0.f);
    case ALGO_POSHIO: {
      float2 r;
      r.x = (p.x > 0.f && inside) ? relax19(x.x, p.x) : x.x - beta * p.x;
      r.y = x.y - beta * p.y;
      return r;
    }
    default:  // FHIO
      return inside ? make_float2(relax19(x.x, p.x), relax19(x.y, p.y))
                    : make_float2(minus12(x.x, p.x), minus12(x.y, p.y));
  }
}

// ---------------------------------------------------------- modulus projections
// applyModAbs with state == NULL (src/gpu/cudaConfig.cu:827-841); amp is
// sqrt(I) precomputed (I <= 0 or NaN -> 0), bit-identical to the per-call sqrtf.
// Where amp is zero (most of a Poisson pattern's far field) the quotient amp/mod
// is that zero, so s * amp gives the same values without the modulus and the
// division, whose zero-dividend case is far slower than its common path
// (2048^2 phase object, 60 % zeros: column pass 29.8 -> 25.1 us).  The one
// difference is the sign of an exact zero: s = (-0, 0) gives (-0, 0) here and
// (0, 0) in the reference, which every later sum treats alike.
__device__ __forceinline__ float2 proj_modabs(float2 s, float amp) {
  if (amp == 0.f) return make_float2(s.x * amp, s.y * amp);
  float mod = hypotf(s.x, s.y);
  if (mod == 0.f) return make_float2(amp, 0.f);
  float rat = amp / mod;
  return make_float2(s.x * rat, s.y * rat);
}
// Noise-tolerant projection, 5-argument applyMod with bsnorm == 1
// (src/gpu/cdi.cu:438-485).  scale = vars.scale, rcolor = vars.rcolor.
__device__ __forceinline__ float2 proj_ccd(float2 s, float inten, float bs, bool has_bs,
                                           int noise, float scale, float rcolor) {
  if (has_bs && bs > 0.5f) return s;
  float mod2 = fmaxf(0.f, inten);
  float src = s.x * s.x + s.y * s.y;
  float maximum = scale * 0.95f;
  if (mod2 >= maximum) mod2 = fmaxf(mod2, src);
  float tol = sqrtf((float)noise + mod2 * rcolor / scale) * scale / rcolor;
  float diff = mod2 - src;
  float val = mod2;
  if (diff > tol) val -= tol;
  else if (diff < -tol) val += tol;
  if (src == 0.f) return make_float2(val, 0.f);
  float sc = sqrtf(fmaxf(val, 0.f) / src);
  return make_float2(sc * s.x, sc * s.y);
}

// ------------------------------------------------------------ block helpers
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// Sum over the CTA in a fixed order; the result is valid in thread 0.
template <int T>
__device__ __forceinline__ double block_sum_d(double v, double* red) {
  v = warp_sum_d(v);
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  if (ln == 0) red[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < T / 32; ++i) r += red[i];
  }
  __syncthreads();
  return r;
}

// ------------------------------------------------ programmatic dependent launch
// The pass kernels are launched with programmatic stream serialisation allowed
// (cudaLaunchAttributeProgrammaticStreamSerialization): each CTA first waits
// until the preceding grid has completed and its writes are visible
// (griddepcontrol.wait: a no-op for a normal launch), then lets the next
// kernel of the stream be scheduled (griddepcontrol.launch_dependents; it
// starts once every CTA of this grid has done so or exited).  The next
// kernel's CTAs thus fill the SMs this grid's last wave leaves idle and wait
// there, instead of being launched after it drains.
__device__ __forceinline__ void pdl_wait_and_release() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

#ifndef CDX_PDL
#define CDX_PDL 1
#endif
// Launch of a register-handoff pass kernel with programmatic dependent launch
// allowed (the kernel waits for its predecessor itself: pdl_wait_and_release).
template <class A>
cudaError_t launch_pdl(void (*kernel)(A), dim3 grid, int block, int smem, cudaStream_t st, const A& a,
                       bool allow = true) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = (CDX_PDL && allow) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

// ------------------------------------------------------------ async copies
// cp.async global -> shared; with `valid` false the destination is zero-filled
// and nothing is read.
__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(src), "r"(valid ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(PENDING) : "memory"); }

// ---------------------------------------------- bulk (TMA) copies to shared
// One thread moves a contiguous run global -> shared with cp.async.bulk
// (the tensor-memory-access engine; 16-byte aligned addresses, size a
// multiple of 16) and the CTA waits on an mbarrier whose transaction count
// the copies complete.  The wait is bounded: past the limit the CTA records
// an error bit (err, may be null) and carries on, so a faulty copy cannot
// hang the GPU; the host reports the bit.
#ifndef CDX_BULK
#define CDX_BULK 1
#endif
constexpr unsigned kBulkSpinLimit = 1u << 22;
// Lines shorter than 1024: measured on one box (graph-captured iterations)
// 384^2 x16 43.2 -> 41.0 us with bulk staging, 192..768 within +-0.4 %, while
// 1024^2 x4, 2048^2 and 4096^2 were 0.3-0.9 % slower than with cp.async by
// every thread, so those lengths keep cp.async.
template <int N>
__host__ __device__ constexpr bool bulk_staging() { return CDX_BULK && N < 1024; }
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bulk_bar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void bulk_expect(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
// warm L2 with `bytes` (a multiple of 16) from a 16-byte aligned global address; no completion
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_wait(uint64_t* bar, int* err) {
  const unsigned b = smem_addr(bar);
  for (unsigned i = 0; i < kBulkSpinLimit; ++i) {
    unsigned ok;
    asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}\n"
                 : "=r"(ok)
                 : "r"(b)
                 : "memory");
    if (ok) return;
  }
  if (err) atomicOr(err, 1);
}

// ------------------------------------------------------------------ layouts
// Element (r, c) of a column-tiled array of `rows` rows with tile width 2^tl.
__device__ __forceinline__ long long tiled_off(int r, int c, int rows, int tl) {
  return ((((long long)(c >> tl)) * rows + r) << tl) + (c & ((1 << tl) - 1));
}

// Element e of a row CTA's L rows -> (row l, column c).  For column-tiled
// global arrays the order is chunk-major: one chunk is the CTA's L rows x one
// tile width, contiguous in HBM, so consecutive threads fill whole sectors.
template <int N, int L, int LOG2L>
__device__ __forceinline__ void row_elem(int e, int tiled, int tl, int& l, int& c) {
  if (tiled && (N & ((1 << tl) - 1)) == 0) {   // whole tiles per row
    const int q = e & ((L << tl) - 1);
    l = q >> tl;
    c = ((e >> (LOG2L + tl)) << tl) + (q & ((1 << tl) - 1));
  } else {
    l = e / N;
    c = e - l * N;
  }
}

// ------------------------------------------------------------ tcgen05 set-up
// Extra dynamic shared memory of the tcgen05 radix-16 passes: the A tiles
// (T/128 x 16 KB), Bm and Bl (4 KB each), 1 KB for the 1024-byte alignment.
template <int N>
constexpr int umma_smem_extra() { return (Geom<N>::T / 128) * kUmmaTileBytes + 2 * kUmmaBBytes + 1024; }

// Allocates the kernel's TMEM (32 columns per 128-butterfly tile), initialises
// the mbarrier and places the operand tiles after `base_bytes` of dynamic
// shared memory.  Every thread of the CTA calls it; it ends with a barrier.
template <int N>
__device__ __forceinline__ void umma_fft_begin(UmmaFft& U, unsigned char* smem_base, int base_bytes, uint64_t* bar,
                                               unsigned* tmem_slot, int* err) {
  constexpr int NT = Geom<N>::T / 128;
  constexpr unsigned COLS = NT * 32 < 32 ? 32 : NT * 32;
  const unsigned s0 = (unsigned)__cvta_generic_to_shared(smem_base);
  const unsigned a = (s0 + (unsigned)base_bytes + 1023u) & ~1023u;
  U.a = a;
  U.bm = a + NT * kUmmaTileBytes;
  U.bl = U.bm + kUmmaBBytes;
  U.bar = (unsigned)__cvta_generic_to_shared(bar);
  U.phase = 0;
  U.err = err;
  if ((threadIdx.x >> 5) == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(
                     (unsigned)__cvta_generic_to_shared(tmem_slot)),
                 "r"(COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (threadIdx.x == 0) {
    umma::mbar_init(U.bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  U.tmem = *tmem_slot;
}

template <int N>
__device__ __forceinline__ void umma_fft_end(const UmmaFft& U) {
  constexpr int NT = Geom<N>::T / 128;
  constexpr unsigned COLS = NT * 32 < 32 ? 32 : NT * 32;
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if ((threadIdx.x >> 5) == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(U.tmem), "r"(COLS) : "memory");
}

// ------------------------------------------------------------------ row pass
// Lines are rows of length N (= number of columns).  Grid: (ceil(rows/L), batch).
template <int N, int MODE, int TC>
__global__ void __launch_bounds__(Geom<N>::T, (TC && Geom<N>::MINB > 2) ? 2 : Geom<N>::MINB) row_pass_kernel(RowArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  extern __shared__ float2 smem[];
  const float2* __restrict__ tw = a.tw;   // read through L1, shared by the SM's CTAs
  float2* buf = smem;
  const int row0 = blockIdx.x * L;
  const int nrows = min(L, a.rows - row0);
  const long long pin = (long long)blockIdx.y * a.in_stride;
  const long long pout = (long long)blockIdx.y * a.out_stride;

  if (a.state && (a.state[blockIdx.y].flags & 4)) return;   // frozen pattern
  // Every global read is an asynchronous copy issued up front: the rows (one
  // group), then in ROW_ITER the L rows of rho (a second group, which lands
  // while the inverse FFT runs).
  const float2* in = a.in + pin;
  constexpr bool iter = MODE == ROW_ITER;
  float2* rho_s = smem + L * G::LD;
  float2* rho = a.rho + (long long)blockIdx.y * a.rho_stride + (long long)row0 * N;
#pragma unroll 4
  for (int e = threadIdx.x; e < L * N; e += T) {
    int l, c;
    row_elem<N, L, G::LOG2L>(e, a.in_tiled, a.tile_log2, l, c);
    const bool ok = l < nrows;
    const int r = row0 + (ok ? l : 0);
    const long long o = a.in_tiled ? tiled_off(r, c, a.rows, a.tile_log2) : (long long)r * N + c;
    cp_async8(buf + G::idx(l, c), in + o, ok);
  }
  cp_commit();
  constexpr int WPR = (N + 31) >> 5;
  uint32_t* mask_s = reinterpret_cast<uint32_t*>(rho_s + L * N);
  if constexpr (iter) {
#pragma unroll 4
    for (int e = threadIdx.x; e < L * N / 2; e += T) {
      const bool ok = (2 * e) / N < nrows;
      cp_async16(rho_s + 2 * e, ok ? rho + 2 * e : rho, ok);
    }
    const uint32_t* mask = a.mask + (long long)blockIdx.y * a.mask_stride + (long long)row0 * WPR;
    for (int w = threadIdx.x; w < L * WPR; w += T) {
      const bool ok = w / WPR < nrows;
      cp_async4(mask_s + w, ok ? mask + w : mask, ok);
    }
  }
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  // tcgen05 passes: TMEM, mbarrier and operand tiles after this mode's buffers
  __shared__ __align__(8) uint64_t um_bar;
  __shared__ unsigned um_tmem;
  UmmaFft U{};
  unsigned char* ub = reinterpret_cast<unsigned char*>(smem);
  if constexpr (TC == 2) umma_fft_begin<N>(U, ub, iter ? G::SMEM_ROW_ITER : G::SMEM_LINES, &um_bar, &um_tmem, a.err);

  if constexpr (!iter) {
    if (a.inv) fft_lines<N, true, TC>(buf, tw, &U, ub);
    else fft_lines<N, false, TC>(buf, tw, &U, ub);
  } else {
    fft_lines<N, true, TC>(buf, tw, &U, ub);
    cp_wait<0>();
    __syncthreads();
    // rho' = IFFT/N, update against rho and the support bits
    for (int e = threadIdx.x; e < L * N; e += T) {
      const int l = e / N, c = e - l * N;
      float2 r = make_float2(0.f, 0.f);
      if (l < nrows) {
        float2 p = buf[G::idx(l, c)];
        p.x *= a.inv_n;
        p.y *= a.inv_n;
        const float2 x = rho_s[e];
        const bool inside = (mask_s[l * WPR + (c >> 5)] >> (c & 31)) & 1u;
        r = apply_update(a.algo, inside, x, p, a.beta);
        rho[e] = r;
      }
      buf[G::idx(l, c)] = r;
    }
    __syncthreads();
    fft_lines<N, false, TC>(buf, tw, &U, ub);
  }
  if constexpr (TC == 2) umma_fft_end<N>(U);
  // store rows
  const float s = a.scale;
  for (int e = threadIdx.x; e < L * N / 2; e += T) {
    int l, c;
    row_elem<N, L, G::LOG2L>(2 * e, a.out_tiled, a.tile_log2, l, c);
    if (l < nrows) {
      float2 u = buf[G::idx(l, c)], v = buf[G::idx(l, c + 1)];
      if (s != 1.f) { u.x *= s; u.y *= s; v.x *= s; v.y *= s; }
      const int r = row0 + l;
      const long long o = a.out_tiled ? tiled_off(r, c, a.rows, a.tile_log2) : (long long)r * N + c;
      *reinterpret_cast<float4*>(a.out + pout + o) = make_float4(u.x, u.y, v.x, v.y);
    }
  }
}

// --------------------------------------------------------------- column pass
// Lines are columns of length N (= number of rows).  Grid: (ceil(cols/L), batch).
// Column-tiled arrays here have tile width L, so the CTA's tile is the
// contiguous block [blockIdx.x * N * L, +N*L) with element t = r*L + l.
template <int N, int MODE, int TC>
__global__ void __launch_bounds__(Geom<N>::T, (TC && Geom<N>::MINB > 2) ? 2 : Geom<N>::MINB) col_pass_kernel(ColArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T, LL = G::LOG2L;
  extern __shared__ float2 smem[];
  __shared__ double red[T / 32];
  const float2* __restrict__ tw = a.tw;
  float2* buf = smem;
  const int c0 = blockIdx.x * L;
  const int ncols = min(L, a.cols - c0);
  const long long C = a.cols;
  const long long tile = (long long)blockIdx.x * N * L;

  // A pattern whose R-factor reached the stop value (flags bit 1, set after the
  // previous column pass) freezes here: this pass and the row pass that follows
  // skip it from now on, leaving rho and W consistent.
  if (a.state) {
    const int f = a.state[blockIdx.y].flags;
    if (f & 6) {
      if ((f & 4) == 0 && threadIdx.x == 0) atomicOr(&a.state[blockIdx.y].flags, 4);
      return;
    }
  }
  // Asynchronous copies issued up front: the column tile (one group), then in
  // COL_ITER the tile's sqrt(I) (and I, beamstop for PROJ_CCD), a second group
  // that lands while the forward FFT runs.
  constexpr bool iter = MODE == COL_ITER;
  const bool ccd = iter && a.proj == PROJ_CCD;
  float* amp_s = reinterpret_cast<float*>(smem + L * G::LD);
  float* int_s = amp_s + L * N;
  float* bs_s = int_s + L * N;
  {
    const float2* in = a.in + (long long)blockIdx.y * a.in_stride;
    if (a.in_tiled) {
#pragma unroll 4
      for (int t = threadIdx.x; t < L * N; t += T) {
        const int r = t >> LL, l = t & (L - 1);
        cp_async8(buf + G::idx(l, r), in + tile + t, true);
      }
    } else {
#pragma unroll 4
      for (int t = threadIdx.x; t < L * N; t += T) {
        const int r = t >> LL, l = t & (L - 1);
        const bool ok = l < ncols;
        cp_async8(buf + G::idx(l, r), in + r * C + c0 + (ok ? l : 0), ok);
      }
    }
  }
  cp_commit();
  const long long aux = (long long)blockIdx.y * a.aux_stride + tile;
  if constexpr (iter) {
    // tiled auxiliaries are padded to whole tiles: always in bounds
#pragma unroll 4
    for (int q = threadIdx.x; q < L * N / 4; q += T) {
      cp_async16(amp_s + 4 * q, a.amp + aux + 4 * q, true);
      if (ccd) {
        cp_async16(int_s + 4 * q, a.inten + aux + 4 * q, true);
        if (a.bs) cp_async16(bs_s + 4 * q, a.bs + aux + 4 * q, true);
      }
    }
  }
  cp_commit();
  cp_wait<1>();
  __syncthreads();
  __shared__ __align__(8) uint64_t um_bar;
  __shared__ unsigned um_tmem;
  UmmaFft U{};
  unsigned char* ub = reinterpret_cast<unsigned char*>(smem);
  if constexpr (TC == 2)
    umma_fft_begin<N>(U, ub, iter ? (ccd ? G::SMEM_COL_CCD : G::SMEM_COL_ITER) : G::SMEM_LINES, &um_bar, &um_tmem,
                      a.err);

  if constexpr (!iter) {
    if (a.inv) fft_lines<N, true, TC>(buf, tw, &U, ub);
    else fft_lines<N, false, TC>(buf, tw, &U, ub);
  } else {
    if (!a.from_psi) fft_lines<N, false, TC>(buf, tw, &U, ub);
    cp_wait<0>();
    __syncthreads();
    // Psi is complete here: optional copy-out, R-factor partial, projection
    double rsum = 0.0;
    for (int t = threadIdx.x; t < L * N; t += T) {
      const int r = t >> LL, l = t & (L - 1);
      if (l < ncols) {
        float2 s = buf[G::idx(l, r)];
        const float amp = amp_s[t];
        if (a.rf_partials) rsum += fabsf(hypotf(s.x, s.y) - amp);
        if (a.proj == PROJ_MODABS) s = proj_modabs(s, amp);
        else s = proj_ccd(s, int_s[t], a.bs ? bs_s[t] : 0.f, a.bs != nullptr,
                          a.noise_level, a.ccd_scale, a.ccd_rcolor);
        if (a.psi_out) a.psi_out[(long long)blockIdx.y * a.psi_stride + r * C + c0 + l] = s;
        buf[G::idx(l, r)] = s;
      }
    }
    if (a.rf_partials) {
      double tsum = block_sum_d<T>(rsum, red);
      if (threadIdx.x == 0) a.rf_partials[(long long)blockIdx.y * gridDim.x + blockIdx.x] = tsum;
    }
    __syncthreads();
    fft_lines<N, true, TC>(buf, tw, &U, ub);
  }
  if constexpr (TC == 2) umma_fft_end<N>(U);
  const float s = a.scale;
  float2* out = a.out + (long long)blockIdx.y * a.out_stride;
  if (a.out_tiled) {
    float4* out4 = reinterpret_cast<float4*>(out + tile);
    for (int e = threadIdx.x; e < L * N / 2; e += T) {
      const int t = 2 * e, r = t >> LL, l = t & (L - 1);
      float2 u = buf[G::idx(l, r)], v = buf[G::idx(l + 1, r)];
      if (s != 1.f) { u.x *= s; u.y *= s; v.x *= s; v.y *= s; }
      out4[e] = make_float4(u.x, u.y, v.x, v.y);
    }
  } else {
    for (int t = threadIdx.x; t < L * N; t += T) {
      const int r = t >> LL, l = t & (L - 1);
      if (l < ncols) {
        float2 v = buf[G::idx(l, r)];
        if (s != 1.f) { v.x *= s; v.y *= s; }
        out[r * C + c0 + l] = v;
      }
    }
  }
}

}  // namespace cdx
