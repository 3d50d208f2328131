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
__device__ __forceinline__ float2 proj_modabs(float2 s, float amp) {
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

// ------------------------------------------------------------------ row pass
// Lines are rows of length N (= number of columns).  Grid: (ceil(rows/L), batch).
template <int N>
__global__ void __launch_bounds__(Geom<N>::T) row_pass_kernel(RowArgs a) {
  constexpr int L = Geom<N>::L, T = Geom<N>::T;
  using LY = Layout<N>;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* buf = smem + N;
  const int row0 = blockIdx.x * L;
  const int nrows = min(L, a.rows - row0);
  const long long poff = (long long)blockIdx.y * a.pat_stride + (long long)row0 * N;

  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  // load rows (two complex per 16-byte access)
  const float4* in4 = reinterpret_cast<const float4*>(a.in + poff);
  for (int e = threadIdx.x; e < L * N / 2; e += T) {
    const int l = (2 * e) / N, c = 2 * e - l * N;
    float4 q = l < nrows ? in4[e] : make_float4(0.f, 0.f, 0.f, 0.f);
    buf[LY::idx(l, c)] = make_float2(q.x, q.y);
    buf[LY::idx(l, c + 1)] = make_float2(q.z, q.w);
  }
  __syncthreads();

  if (a.mode == ROW_FFT) {
    if (a.inv) fft_lines<N, L, T, true>(buf, tw);
    else fft_lines<N, L, T, false>(buf, tw);
  } else {
    fft_lines<N, L, T, true>(buf, tw);
    // rho' = IFFT/N, update against rho and the support bits
    const int wpr = (N + 31) >> 5;
    float2* rho = a.rho + poff;
    const uint32_t* mask = a.mask + (long long)blockIdx.y * a.mask_stride + (long long)row0 * wpr;
    for (int e = threadIdx.x; e < L * N; e += T) {
      const int l = e / N, c = e - l * N;
      if (l < nrows) {
        float2 p = buf[LY::idx(l, c)];
        p.x *= a.inv_n;
        p.y *= a.inv_n;
        const float2 x = rho[e];
        const bool inside = (mask[l * wpr + (c >> 5)] >> (c & 31)) & 1u;
        const float2 r = apply_update(a.algo, inside, x, p, a.beta);
        rho[e] = r;
        buf[LY::idx(l, c)] = r;
      } else {
        buf[LY::idx(l, c)] = make_float2(0.f, 0.f);
      }
    }
    __syncthreads();
    fft_lines<N, L, T, false>(buf, tw);
  }
  // store rows
  float4* out4 = reinterpret_cast<float4*>(a.out + poff);
  const float s = a.scale;
  for (int e = threadIdx.x; e < L * N / 2; e += T) {
    const int l = (2 * e) / N, c = 2 * e - l * N;
    if (l < nrows) {
      float2 u = buf[LY::idx(l, c)], v = buf[LY::idx(l, c + 1)];
      if (s != 1.f) { u.x *= s; u.y *= s; v.x *= s; v.y *= s; }
      out4[e] = make_float4(u.x, u.y, v.x, v.y);
    }
  }
}

// --------------------------------------------------------------- column pass
// Lines are columns of length N (= number of rows).  Grid: (ceil(cols/L), batch).
template <int N>
__global__ void __launch_bounds__(Geom<N>::T) col_pass_kernel(ColArgs a) {
  constexpr int L = Geom<N>::L, T = Geom<N>::T;
  using LY = Layout<N>;
  extern __shared__ float2 smem[];
  __shared__ double red[T / 32];
  float2* tw = smem;
  float2* buf = smem + N;
  const int c0 = blockIdx.x * L;
  const int ncols = min(L, a.cols - c0);
  const long long C = a.cols;
  const long long poff = (long long)blockIdx.y * a.pat_stride + c0;

  for (int i = threadIdx.x; i < N; i += T) tw[i] = a.tw[i];
  const float2* in = a.in + poff;
  for (int e = threadIdx.x; e < L * N; e += T) {
    const int r = e / L, l = e - r * L;
    buf[LY::idx(l, r)] = l < ncols ? in[r * C + l] : make_float2(0.f, 0.f);
  }
  __syncthreads();

  if (a.mode == COL_FFT) {
    if (a.inv) fft_lines<N, L, T, true>(buf, tw);
    else fft_lines<N, L, T, false>(buf, tw);
  } else {
    if (!a.from_psi) fft_lines<N, L, T, false>(buf, tw);
    // Psi is complete here: optional copy-out, R-factor partial, projection
    double rsum = 0.0;
    const long long aoff = (long long)blockIdx.y * a.pat_stride + c0;
    for (int e = threadIdx.x; e < L * N; e += T) {
      const int r = e / L, l = e - r * L;
      if (l < ncols) {
        const long long gi = aoff + r * C + l;
        float2 s = buf[LY::idx(l, r)];
        if (a.psi_out) a.psi_out[gi] = s;
        const float amp = a.amp[gi];
        if (a.rf_partials) rsum += fabsf(hypotf(s.x, s.y) - amp);
        if (a.proj == PROJ_MODABS) s = proj_modabs(s, amp);
        else s = proj_ccd(s, a.inten[gi], a.bs ? a.bs[gi] : 0.f, a.bs != nullptr,
                          a.noise_level, a.ccd_scale, a.ccd_rcolor);
        buf[LY::idx(l, r)] = s;
      }
    }
    if (a.rf_partials) {
      double t = block_sum_d<T>(rsum, red);
      if (threadIdx.x == 0) a.rf_partials[(long long)blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
    __syncthreads();
    fft_lines<N, L, T, true>(buf, tw);
  }
  float2* out = a.out + poff;
  const float s = a.scale;
  for (int e = threadIdx.x; e < L * N; e += T) {
    const int r = e / L, l = e - r * L;
    if (l < ncols) {
      float2 v = buf[LY::idx(l, r)];
      if (s != 1.f) { v.x *= s; v.y *= s; }
      out[r * C + l] = v;
    }
  }
}

}  // namespace cdx
