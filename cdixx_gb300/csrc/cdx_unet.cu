// Warm-start U-Net: layer graph, element-wise kernels (GroupNorm, LeakyReLU,
// loss, Adam) and the C ABI of include/cdx_unet.h.  The convolutions are the
// implicit-GEMM tensor-core kernels of cdx_unet_gemm.cuh.
//
// Flat parameter order (FP32): layers in forward order; per layer the weight
// (conv layout [Cout][KH][KW][Cin]; a transposed convolution stores the
// convolution it is the adjoint of, [Cin_T][2][2][Cout_T]), then GroupNorm
// gamma[C] and beta[C]; the head has weight [4][1][1][base] and bias[4].
// The first convolution sees one input channel.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <type_traits>
#include <cstring>
#include <string>
#include <vector>

#include "cdx.h"
#include "cdx_host.h"
#include "cdx_types.h"
#include "cdx_unet.h"
#include "cdx_unet_gemm.cuh"

namespace cdx {
namespace unet {

#define U_CK(call)                                                                                \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

constexpr int kThreads = 256;

// ------------------------------------------------------------ element-wise kernels
// log(1 + I) / max log(1 + I) per pattern, centred (fftshift), channel 0 of 8
__global__ void k_prep_input(const float* __restrict__ inten, __nv_bfloat16* __restrict__ x, int n) {
  const int b = blockIdx.x;
  const float* I = inten + (long long)b * n * n;
  __shared__ float red[32];
  float mx = 0.f;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) mx = fmaxf(mx, log1pf(fmaxf(I[i], 0.f)));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const float inv = red[0] > 0.f ? 1.f / red[0] : 0.f;
  const int h = n / 2;
  for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
    const int y = i / n, xx = i - y * n;
    const int sy = (y + h) % n, sx = (xx + h) % n;   // centred pixel (y, x) <- FFT-order (y+n/2, x+n/2)
    const float v = log1pf(fmaxf(I[sy * n + sx], 0.f)) * inv;
    __nv_bfloat16* o = x + ((long long)b * n * n + i) * 8;
    o[0] = __float2bfloat16(v);
#pragma unroll
    for (int c = 1; c < 8; ++c) o[c] = __float2bfloat16(0.f);
  }
}

// FP32 weights [co][kh][kw][ci] (real sizes) -> BF16 [co_p][kh][kw][ci_p] and
// transposed [ci_p][kh][kw][co_p], zero-padded
__global__ void k_weights_bf16(const float* __restrict__ w, int co_r, int ci_r, int co_p, int ci_p, int kk,
                               __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wt) {
  const long long total = (long long)co_p * kk * ci_p;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % ci_p);
    const long long t = i / ci_p;
    const int k = (int)(t % kk), co = (int)(t / kk);
    const float v = (co < co_r && ci < ci_r) ? w[((long long)co * kk + k) * ci_r + ci] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16(v);
    wb[i] = b;
    wt[((long long)ci * kk + k) * co_p + co] = b;
  }
}

// sum of wgrad partials over the splits, cropped to the real weight shape
__global__ void k_wgrad_reduce(const float* __restrict__ part, int splits, int co_r, int ci_r, int co_p, int ci_p,
                               int kk, float* __restrict__ grad) {
  const long long total = (long long)co_r * kk * ci_r;
  const long long stride = (long long)co_p * kk * ci_p;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % ci_r);
    const long long t = i / ci_r;
    const int k = (int)(t % kk), co = (int)(t / kk);
    const long long src = ((long long)co * kk + k) * ci_p + ci;
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[z * stride + src];
    grad[i] = s;
  }
}

// GroupNorm statistics: partial sums per (pattern, group, split)
__global__ void k_gn_stats(const float* __restrict__ x, int HW, int C, int G, int split, double* __restrict__ part) {
  const int ng = blockIdx.x, n = ng / G, g = ng - n * G, z = blockIdx.y;
  const int Cg = C / G, tpc = kThreads / Cg;
  const int c = threadIdx.x % Cg, p0 = threadIdx.x / Cg;
  const int pb = (int)((long long)HW * z / split), pe = (int)((long long)HW * (z + 1) / split);
  const float* base = x + (long long)n * HW * C + g * Cg + c;
  float s = 0.f, ss = 0.f;
  for (int p = pb + p0; p < pe; p += tpc) {
    const float v = base[(long long)p * C];
    s += v;
    ss += v * v;
  }
  __shared__ double rs[kThreads], rq[kThreads];
  rs[threadIdx.x] = s;
  rq[threadIdx.x] = ss;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      rs[threadIdx.x] += rs[threadIdx.x + o];
      rq[threadIdx.x] += rq[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[((long long)ng * split + z) * 2] = rs[0];
    part[((long long)ng * split + z) * 2 + 1] = rq[0];
  }
}

__global__ void k_gn_finalize(const double* __restrict__ part, int NG, int split, double count, float* __restrict__ stats) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NG) return;
  double s = 0.0, q = 0.0;
  for (int z = 0; z < split; ++z) {
    s += part[((long long)i * split + z) * 2];
    q += part[((long long)i * split + z) * 2 + 1];
  }
  const double mean = s / count;
  const double var = fmax(q / count - mean * mean, 0.0);
  stats[2 * i] = (float)mean;
  stats[2 * i + 1] = (float)(1.0 / sqrt(var + 1e-5));
}

// y = LeakyReLU(gamma (x - mean) rstd + beta) -> BF16
__global__ void k_gn_apply(const float* __restrict__ x, const float* __restrict__ stats, const float* __restrict__ gamma,
                           const float* __restrict__ beta, int HW, int C, int G, float slope, long long total,
                           __nv_bfloat16* __restrict__ y) {
  const int Cg = C / G;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long long n = i / ((long long)HW * C);
    const int g = c / Cg;
    const float* st = stats + 2 * (n * G + g);
    const float z = (x[i] - st[0]) * st[1] * gamma[c] + beta[c];
    y[i] = __float2bfloat16(z > 0.f ? z : slope * z);
  }
}

// GroupNorm + LeakyReLU backward, pass 1: per (pattern, group, split) sums of
// dz*gamma and dz*gamma*xhat, per channel sums of dz*xhat and dz
__global__ void k_gn_bwd_stats(const float* __restrict__ x, const float* __restrict__ dy, const float* __restrict__ stats,
                               const float* __restrict__ gamma, const float* __restrict__ beta, int HW, int C, int G,
                               int split, float slope, double* __restrict__ part_g, double* __restrict__ part_c) {
  const int ng = blockIdx.x, n = ng / G, g = ng - n * G, z = blockIdx.y;
  const int Cg = C / G, tpc = kThreads / Cg;
  const int c = threadIdx.x % Cg, p0 = threadIdx.x / Cg;
  const int ch = g * Cg + c;
  const int pb = (int)((long long)HW * z / split), pe = (int)((long long)HW * (z + 1) / split);
  const float mean = stats[2 * ng], rstd = stats[2 * ng + 1], ga = gamma[ch], be = beta[ch];
  const long long off = (long long)n * HW * C + ch;
  float s1 = 0.f, s2 = 0.f, dg = 0.f, db = 0.f;
  for (int p = pb + p0; p < pe; p += tpc) {
    const long long i = off + (long long)p * C;
    const float xh = (x[i] - mean) * rstd;
    const float zz = xh * ga + be;
    const float dz = dy[i] * (zz > 0.f ? 1.f : slope);
    s1 += dz * ga;
    s2 += dz * ga * xh;
    dg += dz * xh;
    db += dz;
  }
  __shared__ double r1[kThreads], r2[kThreads], r3[kThreads], r4[kThreads];
  r1[threadIdx.x] = s1;
  r2[threadIdx.x] = s2;
  r3[threadIdx.x] = dg;
  r4[threadIdx.x] = db;
  __syncthreads();
  // channel sums: threads c, c + Cg, c + 2Cg, ... (tree over the tpc threads of a channel)
  for (int o = kThreads / 2; o >= Cg; o >>= 1) {
    if (threadIdx.x < o) {
      r1[threadIdx.x] += r1[threadIdx.x + o];
      r2[threadIdx.x] += r2[threadIdx.x + o];
      r3[threadIdx.x] += r3[threadIdx.x + o];
      r4[threadIdx.x] += r4[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x < Cg) {
    double* pc = part_c + (((long long)n * split + z) * C + ch) * 2;
    pc[0] = r3[threadIdx.x];
    pc[1] = r4[threadIdx.x];
  }
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int k = 0; k < Cg; ++k) {
      a += r1[k];
      b += r2[k];
    }
    part_g[((long long)ng * split + z) * 2] = a;
    part_g[((long long)ng * split + z) * 2 + 1] = b;
  }
}

// pass 2: group sums per (pattern, group) and the gamma/beta gradients
__global__ void k_gn_bwd_finalize(const double* __restrict__ part_g, const double* __restrict__ part_c, int N, int C,
                                  int G, int split, float* __restrict__ gsum, float* __restrict__ dgamma,
                                  float* __restrict__ dbeta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N * G) {
    double a = 0.0, b = 0.0;
    for (int z = 0; z < split; ++z) {
      a += part_g[((long long)i * split + z) * 2];
      b += part_g[((long long)i * split + z) * 2 + 1];
    }
    gsum[2 * i] = (float)a;
    gsum[2 * i + 1] = (float)b;
  }
  if (i < C) {
    double a = 0.0, b = 0.0;
    for (int n = 0; n < N; ++n)
      for (int z = 0; z < split; ++z) {
        const double* pc = part_c + (((long long)n * split + z) * C + i) * 2;
        a += pc[0];
        b += pc[1];
      }
    dgamma[i] = (float)a;
    dbeta[i] = (float)b;
  }
}

// pass 3: dx = rstd (dz gamma - S1/M - xhat S2/M) -> BF16
__global__ void k_gn_bwd_apply(const float* __restrict__ x, const float* __restrict__ dy, const float* __restrict__ stats,
                               const float* __restrict__ gsum, const float* __restrict__ gamma,
                               const float* __restrict__ beta, int HW, int C, int G, float slope, long long total,
                               __nv_bfloat16* __restrict__ dx) {
  const int Cg = C / G;
  const float inv_m = 1.f / ((float)HW * Cg);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % C);
    const long long n = i / ((long long)HW * C);
    const long long ng = n * G + c / Cg;
    const float mean = stats[2 * ng], rstd = stats[2 * ng + 1];
    const float xh = (x[i] - mean) * rstd;
    const float zz = xh * gamma[c] + beta[c];
    const float dz = dy[i] * (zz > 0.f ? 1.f : slope);
    const float v = rstd * (dz * gamma[c] - gsum[2 * ng] * inv_m - xh * gsum[2 * ng + 1] * inv_m);
    dx[i] = __float2bfloat16(v);
  }
}

// head bias: out[m][c] += bias[c], c < 4 (rows of 8 channels)
__global__ void k_bias_add(float* __restrict__ out, const float* __restrict__ bias, long long M) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M * 4; i += (long long)gridDim.x * blockDim.x)
    out[(i >> 2) * 8 + (i & 3)] += bias[i & 3];
}

__device__ __forceinline__ float bce_logits(float z, float t) {
  return fmaxf(z, 0.f) - z * t + log1pf(expf(-fabsf(z)));
}
__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + expf(-z)); }

// per-pixel loss terms of the object (tw = 0) and its twin (tw = 1)
__device__ __forceinline__ float pixel_loss(const float* o, float at, float pt, float st, float ws) {
  float s, c;
  sincosf(pt, &s, &c);
  const float da = o[0] - at, dc = o[1] - c, ds = o[2] - s;
  return da * da + at * (dc * dc + ds * ds) + ws * bce_logits(o[3], st);
}

// partial loss sums per (pattern, split): [object, twin]
__global__ void k_loss_partial(const float* __restrict__ out, const float* __restrict__ amp_t,
                               const float* __restrict__ ph_t, const float* __restrict__ sup_t, int n, int split,
                               float ws, double* __restrict__ part) {
  const int b = blockIdx.x, z = blockIdx.y;
  const int P = n * n;
  const int pb = (int)((long long)P * z / split), pe = (int)((long long)P * (z + 1) / split);
  const long long o = (long long)b * P;
  float l0 = 0.f, l1 = 0.f;
  for (int p = pb + threadIdx.x; p < pe; p += blockDim.x) {
    const int y = p / n, x = p - y * n;
    const int q = ((n - y) % n) * n + (n - x) % n;   // twin pixel -r
    const float* op = out + (o + p) * 8;
    l0 += pixel_loss(op, amp_t[o + p], ph_t[o + p], sup_t[o + p], ws);
    l1 += pixel_loss(op, amp_t[o + q], -ph_t[o + q], sup_t[o + q], ws);
  }
  __shared__ double r0[kThreads], r1[kThreads];
  r0[threadIdx.x] = l0;
  r1[threadIdx.x] = l1;
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      r0[threadIdx.x] += r0[threadIdx.x + s];
      r1[threadIdx.x] += r1[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[((long long)b * split + z) * 2] = r0[0];
    part[((long long)b * split + z) * 2 + 1] = r1[0];
  }
}

// per pattern: the branch with the smaller loss; total = mean over patterns of the per-pixel mean
__global__ void k_loss_select(const double* __restrict__ part, int count, int split, int P, int* __restrict__ twin,
                              double* __restrict__ loss) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tot = 0.0;
  for (int b = 0; b < count; ++b) {
    double a = 0.0, t = 0.0;
    for (int z = 0; z < split; ++z) {
      a += part[((long long)b * split + z) * 2];
      t += part[((long long)b * split + z) * 2 + 1];
    }
    twin[b] = t < a ? 1 : 0;
    tot += (t < a ? t : a) / P;
  }
  *loss = tot / count;
}

// dL/d(head output) for the chosen branch -> BF16 [M][8] (channels 4..7 zero)
__global__ void k_loss_grad(const float* __restrict__ out, const float* __restrict__ amp_t,
                            const float* __restrict__ ph_t, const float* __restrict__ sup_t,
                            const int* __restrict__ twin, int n, int count, float ws, float* __restrict__ dout,
                            __nv_bfloat16* __restrict__ dout_b) {
  const int P = n * n;
  const long long total = (long long)count * P;
  const float sc = 1.f / ((float)P * count);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const int b = (int)(i / P), p = (int)(i - (long long)b * P);
    int q = p;
    float sg = 1.f;
    if (twin[b]) {
      const int y = p / n, x = p - y * n;
      q = ((n - y) % n) * n + (n - x) % n;
      sg = -1.f;
    }
    const long long t = (long long)b * P + q;
    const float at = amp_t[t], pt = sg * ph_t[t], st = sup_t[t];
    float s, c;
    sincosf(pt, &s, &c);
    const float* o = out + i * 8;
    float g[4];
    g[0] = 2.f * (o[0] - at) * sc;
    g[1] = 2.f * at * (o[1] - c) * sc;
    g[2] = 2.f * at * (o[2] - s) * sc;
    g[3] = ws * (sigmoidf_(o[3]) - st) * sc;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dout[i * 4 + k] = g[k];
      dout_b[i * 8 + k] = __float2bfloat16(g[k]);
    }
#pragma unroll
    for (int k = 4; k < 8; ++k) dout_b[i * 8 + k] = __float2bfloat16(0.f);
  }
}

// head bias gradient: sum over pixels of dout[.][c] (fixed order per channel)
__global__ void k_bias_grad(const float* __restrict__ dout, long long M, float* __restrict__ gb) {
  __shared__ double r[kThreads];
  const int c = blockIdx.x;
  double s = 0.0;
  for (long long i = threadIdx.x; i < M; i += blockDim.x) s += dout[i * 4 + c];
  r[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) r[threadIdx.x] += r[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) gb[c] = (float)r[0];
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       long long count, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// network output [b][p][8] -> user [b][4][n][n]
__global__ void k_head_out(const float* __restrict__ o, int P, long long total, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P;
    const int p = (int)(i - b * P);
#pragma unroll
    for (int c = 0; c < 4; ++c) out[(b * 4 + c) * P + p] = o[i * 8 + c];
  }
}
// user layout [b][4][n][n] -> [b][p][8]
__global__ void k_head_in(const float* __restrict__ in, int P, long long total, float* __restrict__ o) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P;
    const int p = (int)(i - b * P);
#pragma unroll
    for (int c = 0; c < 4; ++c) o[i * 8 + c] = in[(b * 4 + c) * P + p];
  }
}

// rho0 (complex, the object frame: the object centred in the array as the
// reference keeps objectWave) and the support from the network output: the
// predicted mask (logit > 0) dilated by `dil` pixels (a square window), since
// HIO tolerates a loose support but not one that cuts into the object
__global__ void k_warm_object(const float* __restrict__ out, int n, int dil, long long total, float2* __restrict__ rho,
                              float* __restrict__ sup) {
  const int P = n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P;
    const int q = (int)(i - b * P);
    const int y = q / n, x = q - y * n;
    const float* o = out + b * 4 * P;
    const float a = fmaxf(o[q], 0.f), c = o[P + q], s = o[2 * P + q], lg = o[3 * P + q];
    bool in = false;
    for (int dy = -dil; dy <= dil && !in; ++dy) {
      const int yy = y + dy;
      if (yy < 0 || yy >= n) continue;
      for (int dx = -dil; dx <= dil; ++dx) {
        const int xx = x + dx;
        if (xx >= 0 && xx < n && o[3 * P + yy * n + xx] > 0.f) {
          in = true;
          break;
        }
      }
    }
    const float r = hypotf(c, s);
    float2 v = make_float2(0.f, 0.f);
    if (lg > 0.f) v = r > 0.f ? make_float2(a * c / r, a * s / r) : make_float2(a, 0.f);
    rho[i] = v;
    sup[i] = in ? 1.f : 0.f;
  }
}

// psi0 = sqrt(I) e^{i arg F}
__global__ void k_warm_psi(const float2* __restrict__ F, const float* __restrict__ inten, long long total,
                           float2* __restrict__ psi) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const float a = sqrtf(fmaxf(inten[i], 0.f));
    const float2 f = F[i];
    const float r = hypotf(f.x, f.y);
    psi[i] = r > 0.f ? make_float2(a * f.x / r, a * f.y / r) : make_float2(a, 0.f);
  }
}

// --------------------------------------------------------------------- host
inline int grid_for(long long total, int threads = kThreads) {
  long long b = (total + threads - 1) / threads;
  const long long cap = sm_count() * 16LL;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

enum { L_CONV = 0, L_CONVT = 1, L_HEAD = 2 };

struct Layer {
  int kind;
  int cin_r, cin_p, cout_r, cout_p;   // layer channels (real / padded)
  int c0;                             // channels of input part 0 (concat)
  int k, s, p;                        // kernel, stride, padding
  int in_h, out_h;                    // spatial sizes
  long long w_off = -1, g_off = -1, b_off = -1, bias_off = -1;
  // underlying convolution weight: [co][k][k][ci] with (co, ci) = (cout, cin) for a
  // convolution and (cin, cout) for a transposed one
  int wco_r, wci_r, wco_p, wci_p;
  __nv_bfloat16 *wb = nullptr, *wt = nullptr;
  int in0 = -1, in1 = -1;             // producer layers (-1: the network input)
  float* pre = nullptr;               // conv output (FP32)
  __nv_bfloat16* act = nullptr;       // activation (BF16)
  float* stats = nullptr;             // mean, rstd per (pattern, group)
  float* dact = nullptr;              // gradient of the activation (FP32)
  __nv_bfloat16* dpre = nullptr;      // gradient of the conv output (BF16)
};

struct Net {
  cdx_unet_config cfg;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  std::vector<Layer> L;
  long long np = 0;
  float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16* x_in = nullptr;
  std::vector<void*> allocs;
  float* wpart = nullptr;
  size_t wpart_cap = 0;
  double *gpart = nullptr, *cpart = nullptr, *lpart = nullptr, *loss = nullptr;
  size_t gpart_cap = 0, cpart_cap = 0;
  float* gsum = nullptr;
  float* dout = nullptr;
  int* twin = nullptr;
  float2* wrk = nullptr;   // warm start scratch
  int* umma_err = nullptr; // set by a tcgen05 tile whose pipeline wait timed out
  int adam_t = 0;
  bool weights_dirty = true;
};

template <typename T>
int dalloc(Net* u, T** p, size_t count) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, count * sizeof(T) + 16);
  if (e != cudaSuccess) return set_error(CDX_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  u->allocs.push_back(q);
  *p = (T*)q;
  return CDX_OK;
}

const __nv_bfloat16* act_of(const Net* u, int idx) { return idx < 0 ? u->x_in : u->L[idx].act; }
int chan_of(const Net* u, int idx) { return idx < 0 ? 8 : u->L[idx].cout_p; }

int build(Net* u) {
  const cdx_unet_config& c = u->cfg;
  const int B = c.batch;
  auto add = [&](int kind, int in0, int in1, int cin_r, int cout_r, int k, int s, int p, int in_h) {
    Layer l{};
    l.kind = kind;
    l.in0 = in0;
    l.in1 = in1;
    l.cin_r = cin_r;
    l.cin_p = in0 < 0 ? 8 : cin_r;
    l.c0 = in1 >= 0 ? chan_of(u, in0) : l.cin_p;
    l.cout_r = cout_r;
    l.cout_p = kind == L_HEAD ? 8 : cout_r;
    l.k = k;
    l.s = s;
    l.p = p;
    l.in_h = in_h;
    l.out_h = kind == L_CONVT ? in_h * 2 : (in_h + 2 * p - k) / s + 1;
    if (kind == L_CONVT) {
      l.wco_r = cin_r; l.wci_r = cout_r; l.wco_p = cin_r; l.wci_p = cout_r;
    } else {
      l.wco_r = cout_r; l.wci_r = in0 < 0 ? 1 : cin_r; l.wco_p = l.cout_p; l.wci_p = l.cin_p;
    }
    l.w_off = u->np;
    u->np += (long long)l.wco_r * k * k * l.wci_r;
    if (kind != L_HEAD) {
      l.g_off = u->np; u->np += cout_r;
      l.b_off = u->np; u->np += cout_r;
    } else {
      l.bias_off = u->np; u->np += 4;
    }
    u->L.push_back(l);
    return (int)u->L.size() - 1;
  };
  std::vector<int> skip(c.levels);
  int h = c.n, ch = c.base;
  int cur = add(L_CONV, -1, -1, 1, ch, 3, 1, 1, h);
  cur = add(L_CONV, cur, -1, ch, ch, 3, 1, 1, h);
  skip[0] = cur;
  for (int l = 1; l < c.levels; ++l) {
    cur = add(L_CONV, cur, -1, ch, ch * 2, 3, 2, 1, h);
    h /= 2;
    ch *= 2;
    cur = add(L_CONV, cur, -1, ch, ch, 3, 1, 1, h);
    skip[l] = cur;
  }
  for (int l = c.levels - 2; l >= 0; --l) {
    const int up = add(L_CONVT, cur, -1, ch, ch / 2, 2, 2, 0, h);
    h *= 2;
    ch /= 2;
    cur = add(L_CONV, up, skip[l], 2 * ch, ch, 3, 1, 1, h);
  }
  add(L_HEAD, cur, -1, ch, 4, 1, 1, 0, h);
  // buffers
  int e;
  if ((e = dalloc(u, &u->params, u->np)) || (e = dalloc(u, &u->grads, u->np)) || (e = dalloc(u, &u->m, u->np)) ||
      (e = dalloc(u, &u->v, u->np)))
    return e;
  if ((e = dalloc(u, &u->x_in, (size_t)B * c.n * c.n * 8))) return e;
  size_t gp = 0, cp = 0, wp = 0;
  for (auto& l : u->L) {
    const size_t px = (size_t)B * l.out_h * l.out_h;
    const size_t wsz = (size_t)l.wco_p * l.k * l.k * l.wci_p;
    if ((e = dalloc(u, &l.wb, wsz)) || (e = dalloc(u, &l.wt, wsz))) return e;
    if ((e = dalloc(u, &l.pre, px * l.cout_p)) || (e = dalloc(u, &l.act, px * l.cout_p)) ||
        (e = dalloc(u, &l.dact, px * l.cout_p)) || (e = dalloc(u, &l.dpre, px * l.cout_p)))
      return e;
    if (l.kind != L_HEAD && (e = dalloc(u, &l.stats, (size_t)B * c.groups * 2))) return e;
    gp = std::max(gp, (size_t)B * c.groups * 64 * 2);
    cp = std::max(cp, (size_t)B * 64 * l.cout_p * 2);
    wp = std::max(wp, (size_t)64 * wsz);
  }
  if ((e = dalloc(u, &u->gpart, gp)) || (e = dalloc(u, &u->cpart, cp)) || (e = dalloc(u, &u->wpart, wp)) ||
      (e = dalloc(u, &u->gsum, (size_t)B * c.groups * 2)) || (e = dalloc(u, &u->lpart, (size_t)B * 64 * 2)) ||
      (e = dalloc(u, &u->loss, 1)) || (e = dalloc(u, &u->dout, (size_t)B * c.n * c.n * 4)) ||
      (e = dalloc(u, &u->twin, (size_t)B)) || (e = dalloc(u, &u->wrk, (size_t)B * c.n * c.n)) ||
      (e = dalloc(u, &u->umma_err, 1)))
    return e;
  u->gpart_cap = gp;
  u->cpart_cap = cp;
  u->wpart_cap = wp;
  return CDX_OK;
}

// He-normal weights from a SplitMix64 stream, GroupNorm gamma 1 / beta 0, head bias 0
void init_params(Net* u, std::vector<float>& h) {
  h.assign(u->np, 0.f);
  uint64_t s = u->cfg.seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  auto next = [&]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto unif = [&]() { return ((next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  for (auto& l : u->L) {
    const long long cnt = (long long)l.wco_r * l.k * l.k * l.wci_r;
    const double fan_in = l.kind == L_CONVT ? (double)l.cin_r : (double)l.k * l.k * l.wci_r;
    const double sd = l.kind == L_HEAD ? std::sqrt(1.0 / fan_in) : std::sqrt(2.0 / fan_in);
    for (long long i = 0; i < cnt; ++i) {
      const double r = std::sqrt(-2.0 * std::log(unif())), t = 6.283185307179586 * unif();
      h[l.w_off + i] = (float)(sd * r * std::cos(t));
    }
    if (l.g_off >= 0)
      for (int i = 0; i < l.cout_r; ++i) h[l.g_off + i] = 1.f;
  }
}

int refresh_weights(Net* u) {
  if (!u->weights_dirty) return CDX_OK;
  for (auto& l : u->L) {
    const long long tot = (long long)l.wco_p * l.k * l.k * l.wci_p;
    k_weights_bf16<<<grid_for(tot), kThreads, 0, u->st>>>(u->params + l.w_off, l.wco_r, l.wci_r, l.wco_p, l.wci_p,
                                                           l.k * l.k, l.wb, l.wt);
  }
  U_CK(cudaGetLastError());
  u->weights_dirty = false;
  return CDX_OK;
}

// the underlying convolution of a layer (for a transposed layer: from its output to its input)
ConvShape conv_shape(const Net* u, const Layer& l, int count) {
  ConvShape s{};
  s.N = count;
  s.KH = s.KW = l.k;
  s.S = l.s;
  s.P = l.p;
  if (l.kind == L_CONVT) {
    s.H = s.W = l.out_h;
    s.Cin = s.C0 = l.cout_p;
    s.Ho = s.Wo = l.in_h;
    s.Cout = l.cin_p;
  } else {
    s.H = s.W = l.in_h;
    s.Cin = l.cin_p;
    s.C0 = l.c0;
    s.Ho = s.Wo = l.out_h;
    s.Cout = l.cout_p;
  }
  (void)u;
  return s;
}

template <int BN, class Op>
int launch_umma(const Op& op, long long M, int NC, int K, int* err, cudaStream_t st) {
  const cudaError_t e = umma::launch_ps<BN, Op>(op, (int)M, NC, K, err, st);
  U_CK(e);
  return CDX_OK;
}

// forward (DGRAD false) or data-gradient GEMM: tcgen05 tiles when the net is
// configured for them, else the mma.sync kernel
template <bool DGRAD>
int launch_gemm(const Net* u, const GemmArgs& a, cudaStream_t st) {
  const ConvShape& s = a.s;
  const long long M = DGRAD ? (long long)s.N * s.H * s.W : (long long)s.N * s.Ho * s.Wo;
  const int NC = DGRAD ? s.Cin : s.Cout;
  const int K = DGRAD ? s.KH * s.KW * s.Cout : s.KH * s.KW * s.Cin;
  if (u->cfg.umma) {
    using Op = typename std::conditional<DGRAD, ConvDgradOp, ConvFwdOp>::type;
    const Op op{a};
    if (NC <= 32) return launch_umma<32>(op, M, NC, K, u->umma_err, st);
    if (NC <= 64) return launch_umma<64>(op, M, NC, K, u->umma_err, st);
    return launch_umma<128>(op, M, NC, K, u->umma_err, st);
  }
  const dim3 grid((unsigned)((M + 127) / 128), (unsigned)((NC + (NC <= 32 ? 31 : 63)) / (NC <= 32 ? 32 : 64)));
  if (NC <= 32) k_conv_gemm<DGRAD, 32><<<grid, 128, 0, st>>>(a);
  else k_conv_gemm<DGRAD, 64><<<grid, 128, 0, st>>>(a);
  U_CK(cudaGetLastError());
  return CDX_OK;
}

int launch_wgrad(Net* u, GemmArgs a, const Layer& l) {
  const ConvShape& s = a.s;
  const long long M = (long long)s.N * s.Ho * s.Wo;
  const int K = s.KH * s.KW * s.Cin;
  const int tx = (K + 63) / 64, ty = (s.Cout + 63) / 64;
  long long splits = (sm_count() * 4LL + tx * ty - 1) / (tx * ty);
  splits = std::max(1LL, std::min(splits, std::min(64LL, (M + 255) / 256)));
  long long mps = (M + splits - 1) / splits;
  mps = (mps + 31) / 32 * 32;
  splits = (M + mps - 1) / mps;
  if ((size_t)(splits * s.Cout * K) > u->wpart_cap) return set_error(CDX_ERR_STATE, "wgrad scratch too small");
  a.out0 = u->wpart;
  a.m_per_split = (int)mps;
  k_conv_wgrad<<<dim3(tx, ty, (unsigned)splits), 128, 0, u->st>>>(a);
  const long long tot = (long long)l.wco_r * l.k * l.k * l.wci_r;
  k_wgrad_reduce<<<grid_for(tot), kThreads, 0, u->st>>>(u->wpart, (int)splits, l.wco_r, l.wci_r, l.wco_p, l.wci_p,
                                                         l.k * l.k, u->grads + l.w_off);
  U_CK(cudaGetLastError());
  return CDX_OK;
}

int gn_split(const Net* u, int HW, int count) {
  const int ng = count * u->cfg.groups;
  int sp = (sm_count() * 4 + ng - 1) / ng;
  sp = std::max(1, std::min(sp, std::min(64, HW / 64 > 0 ? HW / 64 : 1)));
  return sp;
}

int forward(Net* u, const float* inten, int count) {
  const cdx_unet_config& c = u->cfg;
  int e = refresh_weights(u);
  if (e) return e;
  k_prep_input<<<count, 1024, 0, u->st>>>(inten, u->x_in, c.n);
  for (auto& l : u->L) {
    GemmArgs a{};
    a.s = conv_shape(u, l, count);
    if (l.kind == L_CONVT) {
      a.dy = act_of(u, l.in0);
      a.w = l.wt;
      a.out0 = l.pre;
      a.out1 = l.pre;
      if ((e = launch_gemm<true>(u, a, u->st))) return e;
    } else {
      a.x0 = act_of(u, l.in0);
      a.x1 = l.in1 >= 0 ? act_of(u, l.in1) : a.x0;
      a.w = l.wb;
      a.out0 = l.pre;
      if ((e = launch_gemm<false>(u, a, u->st))) return e;
    }
    const long long px = (long long)count * l.out_h * l.out_h;
    if (l.kind == L_HEAD) {
      k_bias_add<<<grid_for(px * 4), kThreads, 0, u->st>>>(l.pre, u->params + l.bias_off, px);
      continue;
    }
    const int HW = l.out_h * l.out_h, sp = gn_split(u, HW, count);
    k_gn_stats<<<dim3(count * c.groups, sp), kThreads, 0, u->st>>>(l.pre, HW, l.cout_p, c.groups, sp, u->gpart);
    k_gn_finalize<<<(count * c.groups + 127) / 128, 128, 0, u->st>>>(u->gpart, count * c.groups, sp,
                                                                      (double)HW * (l.cout_p / c.groups), l.stats);
    k_gn_apply<<<grid_for(px * l.cout_p), kThreads, 0, u->st>>>(l.pre, l.stats, u->params + l.g_off,
                                                                  u->params + l.b_off, HW, l.cout_p, c.groups,
                                                                  c.slope, px * l.cout_p, l.act);
  }
  U_CK(cudaGetLastError());
  return CDX_OK;
}

int backward(Net* u, const float* amp_t, const float* ph_t, const float* sup_t, int count) {
  const cdx_unet_config& c = u->cfg;
  const Layer& head = u->L.back();
  const int P = c.n * c.n;
  for (auto& l : u->L) U_CK(cudaMemsetAsync(l.dact, 0, sizeof(float) * (size_t)count * l.out_h * l.out_h * l.cout_p, u->st));
  const int lsp = std::max(1, std::min(64, (sm_count() * 4 + count - 1) / count));
  k_loss_partial<<<dim3(count, lsp), kThreads, 0, u->st>>>(head.pre, amp_t, ph_t, sup_t, c.n, lsp, c.support_weight,
                                                            u->lpart);
  k_loss_select<<<1, 32, 0, u->st>>>(u->lpart, count, lsp, P, u->twin, u->loss);
  const long long M = (long long)count * P;
  k_loss_grad<<<grid_for(M), kThreads, 0, u->st>>>(head.pre, amp_t, ph_t, sup_t, u->twin, c.n, count,
                                                    c.support_weight, u->dout, head.dpre);
  k_bias_grad<<<4, kThreads, 0, u->st>>>(u->dout, M, u->grads + head.bias_off);
  int e;
  for (int li = (int)u->L.size() - 1; li >= 0; --li) {
    Layer& l = u->L[li];
    const int HW = l.out_h * l.out_h;
    const long long px = (long long)count * HW;
    if (l.kind != L_HEAD) {
      const int sp = gn_split(u, HW, count);
      if ((size_t)count * sp * l.cout_p * 2 > u->cpart_cap) return set_error(CDX_ERR_STATE, "GroupNorm scratch too small");
      k_gn_bwd_stats<<<dim3(count * c.groups, sp), kThreads, 0, u->st>>>(
          l.pre, l.dact, l.stats, u->params + l.g_off, u->params + l.b_off, HW, l.cout_p, c.groups, sp, c.slope,
          u->gpart, u->cpart);
      const int nf = std::max(count * c.groups, l.cout_p);
      k_gn_bwd_finalize<<<(nf + 127) / 128, 128, 0, u->st>>>(u->gpart, u->cpart, count, l.cout_p, c.groups, sp,
                                                              u->gsum, u->grads + l.g_off, u->grads + l.b_off);
      k_gn_bwd_apply<<<grid_for(px * l.cout_p), kThreads, 0, u->st>>>(
          l.pre, l.dact, l.stats, u->gsum, u->params + l.g_off, u->params + l.b_off, HW, l.cout_p, c.groups, c.slope,
          px * l.cout_p, l.dpre);
    }
    GemmArgs a{};
    a.s = conv_shape(u, l, count);
    if (l.kind == L_CONVT) {
      // weight gradient: wgrad of the underlying convolution with X = dz, dY = this layer's input
      a.x0 = l.dpre;
      a.x1 = l.dpre;
      a.dy = act_of(u, l.in0);
      if ((e = launch_wgrad(u, a, l))) return e;
      if (l.in0 >= 0) {
        GemmArgs f{};
        f.s = a.s;
        f.x0 = l.dpre;
        f.x1 = l.dpre;
        f.w = l.wb;
        f.out0 = u->L[l.in0].dact;
        f.accumulate = 1;
        if ((e = launch_gemm<false>(u, f, u->st))) return e;
      }
    } else {
      a.x0 = act_of(u, l.in0);
      a.x1 = l.in1 >= 0 ? act_of(u, l.in1) : a.x0;
      a.dy = l.dpre;
      if ((e = launch_wgrad(u, a, l))) return e;
      if (l.in0 >= 0) {
        GemmArgs d{};
        d.s = a.s;
        d.dy = l.dpre;
        d.w = l.wt;
        d.out0 = u->L[l.in0].dact;
        d.out1 = l.in1 >= 0 ? u->L[l.in1].dact : d.out0;
        d.accumulate = 1;
        if ((e = launch_gemm<true>(u, d, u->st))) return e;
      }
    }
  }
  U_CK(cudaGetLastError());
  return CDX_OK;
}

}  // namespace unet
}  // namespace cdx

using namespace cdx;
using namespace cdx::unet;

struct cdx_unet {
  Net net;
};

extern "C" {

int cdx_unet_config_default(cdx_unet_config* c) {
  if (!c) return set_error(CDX_ERR_ARG, "null config");
  c->n = 256;
  c->levels = 4;
  c->base = 32;
  c->batch = 64;
  c->groups = 8;
  c->slope = 0.01f;
  c->support_weight = 0.1f;
  c->seed = 20260101ull;
  c->umma = 0;
  return CDX_OK;
}

int cdx_unet_create(const cdx_unet_config* c, void* stream, cdx_unet** out) {
  if (!c || !out) return set_error(CDX_ERR_ARG, "null argument");
  *out = nullptr;
  if (c->levels < 2 || c->levels > 8) return set_error(CDX_ERR_ARG, "levels must be in [2, 8]");
  if (c->base < 8 || c->base % 8) return set_error(CDX_ERR_ARG, "base must be a positive multiple of 8");
  if (c->groups < 1 || c->base % c->groups || (kThreads % (c->base / c->groups)) ||
      c->base / c->groups > kThreads)
    return set_error(CDX_ERR_ARG, "groups must divide base (and base/groups divide 256)");
  if (c->n < 16 || c->n % (8 << (c->levels - 1))) return set_error(CDX_ERR_SIZE, "n must be a multiple of 8*2^(levels-1)");
  if (c->batch < 1) return set_error(CDX_ERR_ARG, "batch must be >= 1");
  if (!cdx_size_supported(c->n)) return set_error(CDX_ERR_SIZE, "n is not a supported FFT length");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(CDX_ERR_NOLIB, "no CUDA device");
  }
  cdx_unet* u = new cdx_unet();
  Net* n = &u->net;
  n->cfg = *c;
  if (stream) {
    n->st = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking) != cudaSuccess) {
      delete u;
      return set_error(CDX_ERR_CUDA, "stream create failed");
    }
    n->own_stream = true;
  }
  int e = build(n);
  if (!e) {
    std::vector<float> h;
    init_params(n, h);
    if (cudaMemcpy(n->params, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(n->m, 0, sizeof(float) * n->np) != cudaSuccess ||
        cudaMemset(n->v, 0, sizeof(float) * n->np) != cudaSuccess ||
        cudaMemset(n->grads, 0, sizeof(float) * n->np) != cudaSuccess ||
        cudaMemset(n->umma_err, 0, sizeof(int)) != cudaSuccess)
      e = set_error(CDX_ERR_CUDA, "parameter upload failed");
  }
  if (e) {
    cdx_unet_destroy(u);
    return e;
  }
  *out = u;
  return CDX_OK;
}

void cdx_unet_destroy(cdx_unet* u) {
  if (!u) return;
  Net* n = &u->net;
  if (n->st) cudaStreamSynchronize(n->st);
  for (void* p : n->allocs) cudaFree(p);
  if (n->own_stream && n->st) cudaStreamDestroy(n->st);
  delete u;
}

long long cdx_unet_param_count(const cdx_unet* u) { return u ? u->net.np : -1; }

int cdx_unet_get_params(const cdx_unet* u, float* host, long long count) {
  if (!u || !host || count != u->net.np) return set_error(CDX_ERR_ARG, "bad parameter buffer");
  U_CK(cudaStreamSynchronize(u->net.st));
  U_CK(cudaMemcpy(host, u->net.params, sizeof(float) * count, cudaMemcpyDeviceToHost));
  return CDX_OK;
}

int cdx_unet_set_params(cdx_unet* u, const float* host, long long count) {
  if (!u || !host || count != u->net.np) return set_error(CDX_ERR_ARG, "bad parameter buffer");
  U_CK(cudaStreamSynchronize(u->net.st));
  U_CK(cudaMemcpy(u->net.params, host, sizeof(float) * count, cudaMemcpyHostToDevice));
  u->net.weights_dirty = true;
  return CDX_OK;
}

int cdx_unet_get_grads(const cdx_unet* u, float* host, long long count) {
  if (!u || !host || count != u->net.np) return set_error(CDX_ERR_ARG, "bad gradient buffer");
  U_CK(cudaStreamSynchronize(u->net.st));
  U_CK(cudaMemcpy(host, u->net.grads, sizeof(float) * count, cudaMemcpyDeviceToHost));
  return CDX_OK;
}

static int check_umma(Net* n) {
  int flag = 0;
  U_CK(cudaMemcpyAsync(&flag, n->umma_err, sizeof(int), cudaMemcpyDeviceToHost, n->st));
  U_CK(cudaStreamSynchronize(n->st));
  if (flag) return set_error(CDX_ERR_CUDA, "tensor-core GEMM pipeline wait timed out");
  return CDX_OK;
}

int cdx_unet_forward(cdx_unet* u, const float* intensity, float* out, int count) {
  if (!u || !intensity || !out) return set_error(CDX_ERR_ARG, "null argument");
  if (count < 1 || count > u->net.cfg.batch) return set_error(CDX_ERR_ARG, "count must be in [1, batch]");
  Net* n = &u->net;
  int e = forward(n, intensity, count);
  if (e) return e;
  const int P = n->cfg.n * n->cfg.n;
  k_head_out<<<grid_for((long long)count * P), kThreads, 0, n->st>>>(n->L.back().pre, P, (long long)count * P, out);
  U_CK(cudaGetLastError());
  return check_umma(n);
}

int cdx_unet_loss_backward(cdx_unet* u, const float* intensity, const float* amp_t, const float* phase_t,
                           const float* support_t, int count, double* loss) {
  if (!u || !intensity || !amp_t || !phase_t || !support_t) return set_error(CDX_ERR_ARG, "null argument");
  if (count < 1 || count > u->net.cfg.batch) return set_error(CDX_ERR_ARG, "count must be in [1, batch]");
  Net* n = &u->net;
  int e = forward(n, intensity, count);
  if (e) return e;
  if ((e = backward(n, amp_t, phase_t, support_t, count))) return e;
  if (loss) {
    U_CK(cudaMemcpyAsync(loss, n->loss, sizeof(double), cudaMemcpyDeviceToHost, n->st));
  }
  return check_umma(n);
}

int cdx_unet_adam_step(cdx_unet* u, float lr) {
  if (!u) return set_error(CDX_ERR_ARG, "null network");
  Net* n = &u->net;
  n->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - (float)std::pow((double)b1, n->adam_t), c2 = 1.f - (float)std::pow((double)b2, n->adam_t);
  k_adam<<<grid_for(n->np), kThreads, 0, n->st>>>(n->params, n->grads, n->m, n->v, n->np, lr, b1, b2, 1e-8f, c1, c2);
  U_CK(cudaGetLastError());
  n->weights_dirty = true;
  return CDX_OK;
}

int cdx_unet_warm_start(cdx_unet* u, const float* intensity, const float* out, int count, int dilate, void* psi0,
                        float* support) {
  if (!u || !intensity || !out || !psi0 || !support) return set_error(CDX_ERR_ARG, "null argument");
  if (dilate < 0 || dilate > 16) return set_error(CDX_ERR_ARG, "dilate must be in [0, 16]");
  Net* n = &u->net;
  if (count < 1 || count > n->cfg.batch) return set_error(CDX_ERR_ARG, "count must be in [1, batch]");
  const int N = n->cfg.n;
  const long long tot = (long long)count * N * N;
  k_warm_object<<<grid_for(tot), kThreads, 0, n->st>>>(out, N, dilate, tot, n->wrk, support);
  U_CK(cudaGetLastError());
  int e = cdx_fft2(n->wrk, n->wrk, N, N, count, 0, n->st);
  if (e) return e;
  k_warm_psi<<<grid_for(tot), kThreads, 0, n->st>>>(n->wrk, intensity, tot, (float2*)psi0);
  U_CK(cudaGetLastError());
  U_CK(cudaStreamSynchronize(n->st));
  return CDX_OK;
}

}  // extern "C"
