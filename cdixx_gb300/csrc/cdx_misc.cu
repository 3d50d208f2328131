// Element-wise primitives, shrinkwrap stencil, deterministic reductions and
// initialisation kernels of the CDI path (sm_103a).
#include <algorithm>

#include "cdx_misc.h"
#include "cdx_kernels.cuh"

namespace cdx {

static inline unsigned grid1d(long long n, int t, int cap = 0) {
  if (cap <= 0) cap = sm_count() * 16;
  long long b = (n + t - 1) / t;
  return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// ---------------------------------------------------------------- element-wise
// sqrt(I) as applyModAbs forms it (src/gpu/cudaConfig.cu:830-832): I > 0 -> sqrtf(I), else 0.
__global__ void k_amp(const float* __restrict__ inten, float* __restrict__ amp, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = inten[i];
    amp[i] = v > 0.f ? sqrtf(v) : 0.f;
  }
}
cudaError_t amp_from_pattern(const float* inten, float* amp, long long n, cudaStream_t st) {
  k_amp<<<grid1d(n, 256), 256, 0, st>>>(inten, amp, n);
  return cudaGetLastError();
}

// applyNorm (src/gpu/cudaConfig.cu:425-429)
__global__ void k_scale(float2* __restrict__ x, float s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 v = x[i];
    v.x *= s;
    v.y *= s;
    x[i] = v;
  }
}
cudaError_t scale_complex(float2* x, float s, long long n, cudaStream_t st) {
  k_scale<<<grid1d(n, 256), 256, 0, st>>>(x, s, n);
  return cudaGetLastError();
}

__global__ void k_scale_real(float* __restrict__ x, float s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] *= s;
}
cudaError_t scale_real(float* x, float s, long long n, cudaStream_t st) {
  k_scale_real<<<grid1d(n, 256), 256, 0, st>>>(x, s, n);
  return cudaGetLastError();
}

// cudaConvertFO (src/gpu/cudaConfig.cu:202-212): swap quadrants (even sizes).
template <typename V>
__global__ void k_convert_fo(const V* __restrict__ in, V* __restrict__ out, int rows, int cols, int batch) {
  const long long half = (long long)rows * cols / 2;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < half * batch;
       g += (long long)gridDim.x * blockDim.x) {
    const long long p = g / half, i = g - p * half;
    const int x = (int)(i / cols), y = (int)(i - (long long)x * cols);
    const long long j = (long long)(x + (rows >> 1)) * cols + (y >= (cols >> 1) ? y - (cols >> 1) : y + (cols >> 1));
    const long long base = p * (long long)rows * cols;
    V a = in[base + i], b = in[base + j];
    out[base + i] = b;
    out[base + j] = a;
  }
}
cudaError_t convert_fo_real(const float* in, float* out, int rows, int cols, int batch, cudaStream_t st) {
  k_convert_fo<float><<<grid1d((long long)rows * cols / 2 * batch, 256), 256, 0, st>>>(in, out, rows, cols, batch);
  return cudaGetLastError();
}
cudaError_t convert_fo_complex(const float2* in, float2* out, int rows, int cols, int batch, cudaStream_t st) {
  k_convert_fo<float2><<<grid1d((long long)rows * cols / 2 * batch, 256), 256, 0, st>>>(in, out, rows, cols, batch);
  return cudaGetLastError();
}

// Row-major (rows x cols) -> column-tiled with tile width 2^tl (padding columns
// of the last tile set to 0).  `out_stride` elements between patterns.
__global__ void k_to_tiled(const float* __restrict__ in, float* __restrict__ out, int rows, int cols, int tl,
                           long long out_stride, int batch) {
  const int tw = 1 << tl;
  const int cp = ((cols + tw - 1) >> tl) << tl;
  const long long per = (long long)rows * cp;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < per * batch;
       g += (long long)gridDim.x * blockDim.x) {
    const long long p = g / per, i = g - p * per;
    // i enumerates the tiled array: tile, row, lane
    const long long tile = i / ((long long)rows << tl);
    const long long rem = i - tile * ((long long)rows << tl);
    const int r = (int)(rem >> tl), c = (int)(tile << tl) + (int)(rem & (tw - 1));
    out[p * out_stride + i] = c < cols ? in[p * (long long)rows * cols + (long long)r * cols + c] : 0.f;
  }
}
cudaError_t to_tiled(const float* in, float* out, int rows, int cols, int tl, long long out_stride, int batch,
                     cudaStream_t st) {
  const int cp = ((cols + (1 << tl) - 1) >> tl) << tl;
  k_to_tiled<<<grid1d((long long)rows * cp * batch, 256), 256, 0, st>>>(in, out, rows, cols, tl, out_stride, batch);
  return cudaGetLastError();
}

// Unfused primitives with the reference's element-wise semantics.
__global__ void k_mod_abs(float2* __restrict__ psi, const float* __restrict__ inten, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float v = inten[i];
    psi[i] = proj_modabs(psi[i], v > 0.f ? sqrtf(v) : 0.f);
  }
}
cudaError_t mod_abs(float2* psi, const float* inten, long long n, cudaStream_t st) {
  k_mod_abs<<<grid1d(n, 256), 256, 0, st>>>(psi, inten, n);
  return cudaGetLastError();
}
__global__ void k_mod_ccd(float2* __restrict__ psi, const float* __restrict__ inten, const float* __restrict__ bs,
                          int noise, float scale, float rcolor, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    psi[i] = proj_ccd(psi[i], inten[i], bs ? bs[i] : 0.f, bs != nullptr, noise, scale, rcolor);
}
cudaError_t mod_ccd(float2* psi, const float* inten, const float* bs, int noise, float scale, float rcolor,
                    long long n, cudaStream_t st) {
  k_mod_ccd<<<grid1d(n, 256), 256, 0, st>>>(psi, inten, bs, noise, scale, rcolor, n);
  return cudaGetLastError();
}
__global__ void k_support(float2* __restrict__ rho, const float2* __restrict__ rhop, const float* __restrict__ spt,
                          float thr, float beta, int algo, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    rho[i] = apply_update(algo, spt[i] > thr, rho[i], rhop[i], beta);
}
cudaError_t apply_support(float2* rho, const float2* rhop, const float* spt, float thr, float beta, int algo,
                          long long n, cudaStream_t st) {
  k_support<<<grid1d(n, 256), 256, 0, st>>>(rho, rhop, spt, thr, beta, algo, n);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ supports
// createMask<rect> (src/gpu/cudaConfig.cu:1291-1300): 1 inside [sx,ex) x [sy,ey).
__global__ void k_rect(float* __restrict__ spt, int rows, int cols, int batch, int sx, int sy, int ex, int ey) {
  const long long npx = (long long)rows * cols;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < npx * batch; g += (long long)gridDim.x * blockDim.x) {
    const long long i = g % npx;
    const int x = (int)(i / cols), y = (int)(i - (long long)x * cols);
    spt[g] = (x >= sx && x < ex && y >= sy && y < ey) ? 1.f : 0.f;
  }
}
cudaError_t rect_support(float* spt, int rows, int cols, int batch, int sx, int sy, int ex, int ey, cudaStream_t st) {
  k_rect<<<grid1d((long long)rows * cols * batch, 256), 256, 0, st>>>(spt, rows, cols, batch, sx, sy, ex, ey);
  return cudaGetLastError();
}

// Support bits: bit = spt > threshold of the pattern (the test of cdi.cu:525).
// One warp per 32 columns of one row.
__global__ void k_mask(const float* __restrict__ spt, const PatState* __restrict__ stt, float fixed_thr,
                       uint32_t* __restrict__ bits, int rows, int cols, int batch) {
  const int wpr = (cols + 31) >> 5;
  const long long words = (long long)rows * wpr;
  const long long nw = words * batch;
  const int lane = threadIdx.x & 31;
  for (long long w = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; w < nw;
       w += ((long long)gridDim.x * blockDim.x) >> 5) {
    const long long p = w / words, r = (w - p * words) / wpr, cw = (w - p * words) - r * wpr;
    const int c = (int)cw * 32 + lane;
    const float thr = stt ? stt[p].threshold : fixed_thr;
    bool in = false;
    if (c < cols) in = spt[p * (long long)rows * cols + r * cols + c] > thr;
    const uint32_t b = __ballot_sync(0xffffffffu, in);
    if (lane == 0) bits[w] = b;
  }
}
cudaError_t support_bits(const float* spt, const PatState* st_or_null, float fixed_thr, uint32_t* bits, int rows,
                         int cols, int batch, cudaStream_t st) {
  const long long nw = (long long)rows * ((cols + 31) >> 5) * batch;
  k_mask<<<grid1d(nw * 32, 256), 256, 0, st>>>(spt, st_or_null, fixed_thr, bits, rows, cols, batch);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- shrinkwrap
// Circular separable convolution.  First along the rows index (x), reading rho
// (or |rho|^2 as a real field), then along the columns index (y), writing the
// real support field: |s*v|^2 (Fourier-Gaussian mode, s = rows*cols restores
// the unnormalised IFFT scale of the reference) or Re v (|rho|^2 mode).
constexpr int kBlurRadMax = 64;   // largest stencil radius (host-checked)
constexpr int kBlurTX = 64;       // output rows per CTA of the x pass

__device__ __forceinline__ int wrap(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// x pass: CTA = 32 columns x kBlurTX rows of outputs; the rows it needs (with
// the periodic halo of `rad` on both sides) are staged in shared memory sized
// for this radius (dynamic), so small radii keep more CTAs per SM.
__global__ void __launch_bounds__(256) k_blur_x(const float2* __restrict__ rho, float2* __restrict__ tmp,
                                                const float* __restrict__ w, int rad, int rows, int cols,
                                                int mod2_first, const PatState* __restrict__ stt) {
  if (stt[blockIdx.z].flags & 6) return;   // converged patterns keep their support
  extern __shared__ float2 s[];            // (kBlurTX + 2 rad) x 32, then the 2 rad + 1 weights
  float* ws = reinterpret_cast<float*>(s + (kBlurTX + 2 * rad) * 32);
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int y = blockIdx.x * 32 + tx;
  const int x0 = blockIdx.y * kBlurTX;
  const long long npx = (long long)rows * cols;
  const float2* src = rho + blockIdx.z * npx;
  for (int i = threadIdx.x; i <= 2 * rad; i += 256) ws[i] = w[i];
  const int nload = kBlurTX + 2 * rad;
  for (int j = ty; j < nload; j += 8) {
    float2 v = make_float2(0.f, 0.f);
    if (y < cols) v = src[(long long)wrap(x0 - rad + j, rows) * cols + y];
    if (mod2_first) v = make_float2(v.x * v.x + v.y * v.y, 0.f);
    s[j * 32 + tx] = v;
  }
  __syncthreads();
  if (y >= cols) return;
  // 8 outputs per thread (rows ty, ty+8, ..., ty+56) accumulated together
  float ax[8], ay[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) ax[q] = ay[q] = 0.f;
  for (int d = 0; d <= 2 * rad; ++d) {
    const float wd = ws[d];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float2 v = s[(ty + 8 * q + d) * 32 + tx];
      ax[q] = fmaf(wd, v.x, ax[q]);
      ay[q] = fmaf(wd, v.y, ay[q]);
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int k = ty + 8 * q;
    if (x0 + k < rows) tmp[blockIdx.z * npx + (long long)(x0 + k) * cols + y] = make_float2(ax[q], ay[q]);
  }
}

// y pass: each warp filters whole 256-column row segments on its own (rows
// blockIdx.y*8 + warp, stepping by gridDim.y*8), the segment and its periodic
// halo staged in the warp's slice of shared memory; no block barrier in the
// row loop.  Writes the support field and per-CTA max / sum partials.
__global__ void __launch_bounds__(256) k_blur_y(const float2* __restrict__ tmp, float* __restrict__ spt,
                                                const float* __restrict__ w, int rad, int rows, int cols,
                                                int mod2_first, float s, float* __restrict__ pmax,
                                                double* __restrict__ psum, const PatState* __restrict__ stt) {
  if (stt[blockIdx.z].flags & 6) return;
  extern __shared__ float2 seg_all[];      // 8 x (256 + 2 rad), then the weights
  const int seglen = 256 + 2 * rad;
  float* ws = reinterpret_cast<float*>(seg_all + 8 * seglen);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float2* seg = seg_all + wid * seglen;
  const long long npx = (long long)rows * cols;
  const long long p = blockIdx.z;
  const float2* src = tmp + p * npx;
  float* out = spt + p * npx;
  for (int i = threadIdx.x; i <= 2 * rad; i += 256) ws[i] = w[i];
  __syncthreads();
  const int y0 = blockIdx.x * 256;
  float m = 0.f;   // findMax initialises with 0 (src/gpu/cub_wrap.cu:88-92)
  double acc = 0.0;
  for (int r = blockIdx.y * 8 + wid; r < rows; r += gridDim.y * 8) {
    __syncwarp();
    for (int j = lane; j < seglen; j += 32) seg[j] = src[(long long)r * cols + wrap(y0 - rad + j, cols)];
    __syncwarp();
    float ax[8], ay[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) ax[q] = ay[q] = 0.f;
    for (int d = 0; d <= 2 * rad; ++d) {
      const float wd = ws[d];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float2 v = seg[lane + 32 * q + d];
        ax[q] = fmaf(wd, v.x, ax[q]);
        ay[q] = fmaf(wd, v.y, ay[q]);
      }
    }
    float racc = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int y = y0 + lane + 32 * q;
      if (y >= cols) continue;
      float o;
      if (mod2_first) {
        o = ax[q];
      } else {
        const float sx = ax[q] * s, sy = ay[q] * s;
        o = sx * sx + sy * sy;
      }
      out[(long long)r * cols + y] = o;
      m = fmaxf(m, o);   // a NaN input is dropped by fmaxf; the finaliser checks the sum
      racc += o;
    }
    acc += (double)racc;
  }
  __shared__ float sm[32];
  __shared__ double sd[32];
  m = warp_max_f(m);
  acc = warp_sum_d(acc);
  if (lane == 0) { sm[wid] = m; sd[wid] = acc; }
  __syncthreads();
  if (threadIdx.x == 0) {
    float mm = 0.f;
    double ss = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { mm = fmaxf(mm, sm[i]); ss += sd[i]; }
    const int nb = gridDim.x * gridDim.y, b = blockIdx.y * gridDim.x + blockIdx.x;
    pmax[p * nb + b] = mm;
    psum[p * nb + b] = ss;
  }
}

// Threshold logic of the shrinkwrap block (src/post_gpu/cdi.cc:330-337):
// maxs = findMax; first time avg = findSum*4/rows/cols; maxs = min(maxs, 5*avg);
// threshold = maxs*shrinkThreshold.  |rho|^2 mode: threshold = max*shrinkThreshold.
// One warp per pattern: lane i folds partials i, i + 32, ... in order, then a
// butterfly across the lanes (a fixed order, so the same sum on every device).
__global__ void k_shrink_finalize(const float* __restrict__ pmax, const double* __restrict__ psum, int nblk,
                                  PatState* __restrict__ stt, int rows, int cols, int mod2_first,
                                  double shrink_threshold) {
  const int p = blockIdx.x;
  if (stt[p].flags & 6) return;   // converged: no partials this time
  float m = 0.f;
  double s = 0.0;
  for (int i = threadIdx.x; i < nblk; i += 32) { m = fmaxf(m, pmax[p * nblk + i]); s += psum[p * nblk + i]; }
  m = warp_max_f(m);
  s = warp_sum_d(s);
  if (threadIdx.x != 0) return;
  PatState& S = stt[p];
  S.maxv = m;
  S.sum = (float)s;
  if (s != s) S.flags |= 1;
  if (!mod2_first) {
    if (S.avg == 0.f) S.avg = (float)s * 4.f / (float)rows / (float)cols;
    if (S.avg * 5.f < m) m = S.avg * 5.f;
  }
  if (fabsf(m) < 1e-7f || m != m) S.flags |= 1;
  S.threshold = (float)((double)m * shrink_threshold);
}

cudaError_t shrinkwrap(const float2* rho, float2* tmp, float* spt, const float* wx, int radx, const float* wy,
                       int rady, int rows, int cols, int batch, int mod2_first, float s, float* pmax, double* psum,
                       int nblk, PatState* stt, double shrink_threshold, cudaStream_t st) {
  if (radx > kBlurRadMax || rady > kBlurRadMax || radx < 0 || rady < 0) return cudaErrorInvalidValue;
  const size_t smx = sizeof(float2) * (kBlurTX + 2 * radx) * 32 + sizeof(float) * (2 * radx + 1);
  k_blur_x<<<dim3((cols + 31) / 32, (rows + kBlurTX - 1) / kBlurTX, batch), 256, smx, st>>>(rho, tmp, wx, radx, rows,
                                                                                            cols, mod2_first, stt);
  // y pass: gx segments per row, gy groups of 8 rows; gx*gy <= nblk partials per pattern
  const int gx = (cols + 255) / 256;
  const int gy = std::max(1, std::min((rows + 7) / 8, nblk / gx));
  if (gx * gy > nblk) return cudaErrorInvalidValue;
  const size_t smy = sizeof(float2) * 8 * (256 + 2 * rady) + sizeof(float) * (2 * rady + 1);
  k_blur_y<<<dim3(gx, gy, batch), 256, smy, st>>>(tmp, spt, wy, rady, rows, cols, mod2_first, s, pmax, psum, stt);
  k_shrink_finalize<<<batch, 32, 0, st>>>(pmax, psum, gx * gy, stt, rows, cols, mod2_first, shrink_threshold);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- reductions
// Per pattern: sum sqrt(I) (R-factor denominator).
__global__ void k_sum_real(const float* __restrict__ x, long long npx, double* __restrict__ part, int nblk) {
  const long long p = blockIdx.y;
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npx; i += (long long)nblk * blockDim.x)
    acc += (double)x[p * npx + i];
  __shared__ double red[8];
  double t = block_sum_d<256>(acc, red);
  if (threadIdx.x == 0) part[p * nblk + blockIdx.x] = t;
}
// The closing sums of a run in one pass over the final Psi and I: the residual
// of src/post_gpu/cdi.cc:413-421, sum (|Psi|^2 - I)^2 over I < 0.99, and the
// R-factor numerator sum | |Psi| - sqrt(I) |.  Each thread takes two adjacent
// pixels per step (one 16-byte load of Psi, one 8-byte load of I) with the
// loop unrolled, so a CTA of 1024 threads per SM keeps enough loads in flight
// to stream the pattern at HBM speed.  Partials per pattern: [0, nblk) the
// residual, [nblk, 2 nblk) the R-factor; the order of every sum is fixed.
__device__ __forceinline__ void res_rdiff_px(float2 v, float I, double& r, double& d) {
  float q = v.x * v.x + v.y * v.y;
  q = I < 0.99f ? q - I : 0.f;
  r += (double)q * (double)q;
  d += (double)fabsf(hypotf(v.x, v.y) - (I > 0.f ? sqrtf(I) : 0.f));
}
constexpr int kResThreads = 1024;
__global__ void __launch_bounds__(kResThreads) k_res_rdiff(const float2* __restrict__ psi, const float* __restrict__ inten,
                                                           long long npx, double* __restrict__ part, int nblk) {
  const long long p = blockIdx.y;
  const float2* ps = psi + p * npx;
  const float* in = inten + p * npx;
  double r0 = 0.0, r1 = 0.0, d0 = 0.0, d1 = 0.0;
  const long long step = 2LL * nblk * kResThreads;
#pragma unroll 4
  for (long long i = 2LL * (blockIdx.x * (long long)kResThreads + threadIdx.x); i < npx; i += step) {
    const float4 v = *reinterpret_cast<const float4*>(ps + i);   // npx even: pixels i, i + 1
    const float2 I = *reinterpret_cast<const float2*>(in + i);
    res_rdiff_px(make_float2(v.x, v.y), I.x, r0, d0);
    res_rdiff_px(make_float2(v.z, v.w), I.y, r1, d1);
  }
  __shared__ double red[kResThreads / 32];
  const double tr = block_sum_d<kResThreads>(r0 + r1, red);
  const double td = block_sum_d<kResThreads>(d0 + d1, red);
  if (threadIdx.x == 0) {
    part[p * 2 * nblk + blockIdx.x] = tr;
    part[p * 2 * nblk + nblk + blockIdx.x] = td;
  }
}
__global__ void k_res_rdiff_finalize(const double* __restrict__ part, int nblk, PatState* __restrict__ stt) {
  const int p = blockIdx.x;
  double r = 0.0, d = 0.0;
  for (int i = threadIdx.x; i < nblk; i += 32) {
    r += part[p * 2 * nblk + i];
    d += part[p * 2 * nblk + nblk + i];
  }
  r = warp_sum_d(r);
  d = warp_sum_d(d);
  if (threadIdx.x == 0) {
    stt[p].residual = r;
    stt[p].rfactor = stt[p].amp_sum > 0.0 ? d / stt[p].amp_sum : 0.0;
  }
}

// Fixed-order final sums.  what: 0 amp_sum, 1 residual, 2 rfactor (= sum / amp_sum).
// For an in-loop R-factor (iter >= 0) a pattern with R <= stop gets flags bit 1
// and conv_iter = iter + 1 (it still completes this iteration); stop is the
// pattern's own PatState::stop when set, else the run's `stop` (> 0 to act).
// With plateau > 0 a pattern whose R-factor has not fallen below (1 - tol)
// times its last improvement for `plateau` iterations freezes the same way.
// One warp per pattern, lane-strided sums and a butterfly across the lanes (fixed order).
__global__ void k_finalize_sum(const double* __restrict__ part, int nblk, PatState* __restrict__ stt, int what,
                               double stop, int iter, int plateau, float tol) {
  const int p = blockIdx.x;
  if (iter >= 0 && (stt[p].flags & 6)) return;   // already converged: partials are stale
  double s = 0.0;
  for (int i = threadIdx.x; i < nblk; i += 32) s += part[p * nblk + i];
  s = warp_sum_d(s);
  if (threadIdx.x != 0) return;
  if (what == 0) stt[p].amp_sum = s;
  else if (what == 1) stt[p].residual = s;
  else {
    const double r = stt[p].amp_sum > 0.0 ? s / stt[p].amp_sum : 0.0;
    stt[p].rfactor = r;
    if (iter >= 0 && r < stt[p].rmin) stt[p].rmin = r;
    const double sp = stt[p].stop > 0.0 ? stt[p].stop : stop;
    if (iter >= 0 && sp > 0.0 && r <= sp) {
      stt[p].flags |= 2;
      stt[p].conv_iter = iter + 1;
    } else if (iter >= 0 && plateau > 0) {
      if (r < stt[p].rbest * (1.0 - (double)tol)) {
        stt[p].rbest = r;
        stt[p].best_iter = iter;
      } else if (iter - stt[p].best_iter >= plateau) {
        stt[p].flags |= 2 | 8;
        stt[p].conv_iter = iter + 1;
      }
    }
  }
}

cudaError_t pattern_amp_sum(const float* amp, long long npx, int batch, double* part, int nblk, PatState* stt,
                            cudaStream_t st) {
  k_sum_real<<<dim3(nblk, batch), 256, 0, st>>>(amp, npx, part, nblk);
  k_finalize_sum<<<batch, 32, 0, st>>>(part, nblk, stt, 0, 0.0, -1, 0, 0.f);
  return cudaGetLastError();
}
cudaError_t residual_rfactor(const float2* psi, const float* inten, long long npx, int batch, double* part, int nblk,
                             PatState* stt, cudaStream_t st) {
  if (npx % 2) return cudaErrorInvalidValue;
  k_res_rdiff<<<dim3(nblk, batch), kResThreads, 0, st>>>(psi, inten, npx, part, nblk);
  k_res_rdiff_finalize<<<batch, 32, 0, st>>>(part, nblk, stt);
  return cudaGetLastError();
}
cudaError_t rfactor_from_partials(const double* part, int nblk, int batch, PatState* stt, double stop, int iter,
                                  int plateau, float tol, cudaStream_t st) {
  k_finalize_sum<<<batch, 32, 0, st>>>(part, nblk, stt, 2, stop, iter, plateau, tol);
  return cudaGetLastError();
}

// Start of phaseRetrieve: avg and the flags are locals of the call (cdi.cc:315).
__global__ void k_run_begin(PatState* stt, int batch) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < batch) {
    stt[p].avg = 0.f;
    stt[p].flags = 0;
    stt[p].conv_iter = -1;
    stt[p].rmin = __longlong_as_double(0x7ff0000000000000LL);   // +inf
    stt[p].rbest = stt[p].rmin;
    stt[p].best_iter = 0;
  }
}
cudaError_t run_begin(PatState* stt, int batch, cudaStream_t st) {
  k_run_begin<<<(batch + 127) / 128, 128, 0, st>>>(stt, batch);
  return cudaGetLastError();
}
__global__ void k_state_init(PatState* stt, int batch, float thr) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < batch) {
    PatState z = {};
    z.threshold = thr;
    stt[p] = z;
  }
}
cudaError_t state_init(PatState* stt, int batch, float thr, cudaStream_t st) {
  k_state_init<<<(batch + 127) / 128, 128, 0, st>>>(stt, batch, thr);
  return cudaGetLastError();
}

// ------------------------------------------------------------ random start
// createWaveFront(I, 0, Psi, 1) then applyRandomPhase (src/gpu/cudaConfig.cu:710-732,
// src/gpu/cdi.cu:486-502): Psi = sqrt(max(0,I)) e^{i pi b}, b a fair coin per pixel;
// pixels with beamstop > threshold are zeroed.  The coin is a counter-based hash
// of (seed, pattern, pixel) (SplitMix64 finaliser), not curand's MRG32k3a stream.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
__global__ void k_random_start(const float* __restrict__ inten, const float* __restrict__ bs, float bs_thr,
                               float2* __restrict__ psi, long long npx, int batch, unsigned long long seed) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < npx * batch; g += (long long)gridDim.x * blockDim.x) {
    const float I = inten[g];
    const float mod = sqrtf(fmaxf(0.f, I));
    if (bs && bs[g] > bs_thr) { psi[g] = make_float2(0.f, 0.f); continue; }
    const uint64_t h = mix64(seed * 0x9e3779b97f4a7c15ULL + (uint64_t)g + 1);
    const float u = (float)((h >> 40) + 1) * (1.0f / 16777216.0f);   // (0,1]
    const float ph = (u > 0.5f) ? (float)M_PI : 0.f;
    float s, c;
    sincosf(ph, &s, &c);
    psi[g] = make_float2(mod * c, mod * s);
  }
}
cudaError_t random_start(const float* inten, const float* bs, float bs_thr, float2* psi, long long npx, int batch,
                         unsigned long long seed, cudaStream_t st) {
  k_random_start<<<grid1d(npx * batch, 256), 256, 0, st>>>(inten, bs, bs_thr, psi, npx, batch, seed);
  return cudaGetLastError();
}

cudaError_t misc_prepare() {
  // the x pass of the largest radius needs more than the default 48 KB
  const int smx = (int)(sizeof(float2) * (kBlurTX + 2 * kBlurRadMax) * 32 + sizeof(float) * (2 * kBlurRadMax + 1));
  return cudaFuncSetAttribute(k_blur_x, cudaFuncAttributeMaxDynamicSharedMemorySize, smx);
}

// ---------------------------------------------------------------------- PRTF
// One PRTF step per pattern (cdi.cc:355-380): with the ER update of
// applySupport (inside: x + 1.9 (rho' - x), outside: 0),
//   first step:  gamma0 = ER(0, rho'), cache = gamma0 * gamma0
//   later steps: cache = ER(cache, rho') * conj(gamma0)
// and the complex sum of cache (fixed-order partials per CTA, then per pattern):
// phi0 = -arg(sum)/2 at the first step, theta = phi0 + arg(sum) afterwards.
__global__ void k_prtf_step(const float2* __restrict__ rhop, const uint32_t* __restrict__ bits, int rows, int cols,
                            float2* __restrict__ cache, float2* __restrict__ gamma0, int first,
                            double* __restrict__ part, int nblk, const PatState* __restrict__ stt) {
  const long long p = blockIdx.y;
  const long long npx = (long long)rows * cols;
  const int wpr = (cols + 31) >> 5;
  double sr = 0.0, si = 0.0;
  if (!(stt[p].flags & 4)) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < npx; i += (long long)nblk * blockDim.x) {
      const long long g = p * npx + i;
      const int r = (int)(i / cols), c = (int)(i - (long long)r * cols);
      const bool inside = (bits[p * rows * wpr + (long long)r * wpr + (c >> 5)] >> (c & 31)) & 1u;
      const float2 q = rhop[g];
      float2 v;
      if (first) {
        const float2 g0 = inside ? make_float2(relax19(0.f, q.x), relax19(0.f, q.y)) : make_float2(0.f, 0.f);
        gamma0[g] = g0;
        v = cmul(g0, g0);
      } else {
        const float2 x = cache[g];
        const float2 e = inside ? make_float2(relax19(x.x, q.x), relax19(x.y, q.y)) : make_float2(0.f, 0.f);
        const float2 g0 = gamma0[g];
        v = cmul(e, make_float2(g0.x, -g0.y));
      }
      cache[g] = v;
      sr += v.x;
      si += v.y;
    }
  }
  __shared__ double rr[8], ri[8];
  sr = warp_sum_d(sr);
  si = warp_sum_d(si);
  if ((threadIdx.x & 31) == 0) { rr[threadIdx.x >> 5] = sr; ri[threadIdx.x >> 5] = si; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += rr[w]; b += ri[w]; }
    part[(p * nblk + blockIdx.x) * 2] = a;
    part[(p * nblk + blockIdx.x) * 2 + 1] = b;
  }
}

__global__ void k_prtf_phase(const double* __restrict__ part, int nblk, PrtfState* __restrict__ ps, int first) {
  const int p = blockIdx.x;
  if (threadIdx.x != 0) return;
  double a = 0.0, b = 0.0;
  for (int i = 0; i < nblk; ++i) { a += part[(p * nblk + i) * 2]; b += part[(p * nblk + i) * 2 + 1]; }
  // findSum returns a float complex; phi0 and phi are Real (float) in phaseRetrieve
  const float ang = atan2f((float)b, (float)a);
  if (first) {
    ps[p].phi0 = -ang / 2;
    ps[p].theta = ps[p].phi0;
  } else {
    ps[p].theta = ps[p].phi0 + ang;
  }
}

cudaError_t prtf_step(const float2* rhop, const uint32_t* bits, int rows, int cols, int batch, float2* cache,
                      float2* gamma0, int first, double* part, int nblk, PrtfState* ps, const PatState* stt,
                      cudaStream_t st) {
  k_prtf_step<<<dim3(nblk, batch), 256, 0, st>>>(rhop, bits, rows, cols, cache, gamma0, first, part, nblk, stt);
  k_prtf_phase<<<batch, 32, 0, st>>>(part, nblk, ps, first);
  return cudaGetLastError();
}

// addPhase (src/gpu/cudaConfig.cu:876-887): map += (b/|b|) e^{i theta} where
// |b| > 1e-6; on the first step also the |b| > 1e-6 mask (bitMap, cdi.cc:363).
__global__ void k_prtf_accum(const float2* __restrict__ b, float2* __restrict__ map, float* __restrict__ mask,
                             long long npx, int batch, const PrtfState* __restrict__ ps,
                             const PatState* __restrict__ stt) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < npx * batch;
       g += (long long)gridDim.x * blockDim.x) {
    const long long p = g / npx;
    if (stt[p].flags & 4) continue;
    const float2 v = b[g];
    const float mod = hypotf(v.x, v.y);
    if (mask) mask[g] = mod > 1e-6f ? 1.f : 0.f;
    if (mod > 1e-6f) {
      const float r = v.x / mod, i = v.y / mod;
      float s, c;
      sincosf(ps[p].theta, &s, &c);
      float2 m = map[g];
      m.x += r * c - i * s;
      m.y += r * s + i * c;
      map[g] = m;
    }
  }
}

cudaError_t prtf_accum(const float2* psi_proj, float2* map, float* mask_or_null, long long npx, int batch,
                       const PrtfState* ps, const PatState* stt, cudaStream_t st) {
  k_prtf_accum<<<grid1d(npx * batch, 256), 256, 0, st>>>(psi_proj, map, mask_or_null, npx, batch, ps, stt);
  return cudaGetLastError();
}

// cart2polar_kernel + edgeReduce on the centred image (cudaConvertFO of the
// FFT-order field): for radius r < rows/2, the sum over 2*cols angles, in
// angle order and in float like edgeReduce, of the bilinear sample at
// (r cos t, r sin t) about the centre (rows/2, cols/2).  The image is the
// mask (float) or |map| * inv_count.
__device__ __forceinline__ float prtf_pixel(const float* mask, const float2* map, float inv_count, int rows, int cols,
                                            int x, int y) {
  const int fx = (x + (rows >> 1)) % rows, fy = (y + (cols >> 1)) % cols;   // centred -> FFT order
  const long long i = (long long)fx * cols + fy;
  if (mask) return mask[i];
  const float2 m = map[i];
  return hypotf(m.x, m.y) * inv_count;
}
__global__ void k_prtf_polar(const float* __restrict__ mask, const float2* __restrict__ map, float inv_count,
                             int rows, int cols, float* __restrict__ out) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const long long p = blockIdx.y;
  if (r >= (rows >> 1)) return;
  const long long npx = (long long)rows * cols;
  const float* mk = mask ? mask + p * npx : nullptr;
  const float2* mp = map ? map + p * npx : nullptr;
  const int nang = cols << 1;
  float acc = 0.f;
  for (int a = 0; a < nang; ++a) {
    float s, c;
    sincosf((float)(a * (2.0 * 3.14159265358979323846 / nang)), &s, &c);   // x * (2.0f*M_PI/cuda_row): double
    float x = r * c + (rows >> 1), y = r * s + (cols >> 1);
    const int x0 = (int)floorf(x), y0 = (int)floorf(y);
    const float fx = x - x0, fy = y - y0;
    float v = 0.f;
    if (!(x0 < 0 || x0 + 1 >= rows || y0 < 0 || y0 + 1 >= cols)) {
      const float v00 = prtf_pixel(mk, mp, inv_count, rows, cols, x0, y0);
      const float v01 = prtf_pixel(mk, mp, inv_count, rows, cols, x0, y0 + 1);
      const float v10 = prtf_pixel(mk, mp, inv_count, rows, cols, x0 + 1, y0);
      const float v11 = prtf_pixel(mk, mp, inv_count, rows, cols, x0 + 1, y0 + 1);
      v = (1 - fx) * (1 - fy) * v00 + (1 - fx) * fy * v01 + fx * (1 - fy) * v10 + fx * fy * v11;
    }
    acc += v;
  }
  out[p * (rows >> 1) + r] = acc;
}

cudaError_t prtf_polar(const float* mask, const float2* map, float inv_count, int rows, int cols, int batch,
                       float* out, cudaStream_t st) {
  k_prtf_polar<<<dim3(((rows >> 1) + 127) / 128, batch), 128, 0, st>>>(mask, map, inv_count, rows, cols, out);
  return cudaGetLastError();
}

}  // namespace cdx
