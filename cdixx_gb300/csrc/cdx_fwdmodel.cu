// Seeded synthetic diffraction patterns on the GPU (the forward model that
// generates warm-start training pairs).  No reference counterpart: the
// reference simulates from image files (src/post_gpu/cdi.cc:161-200).
//
// Random numbers are counter based: u(seed, pattern, stream, i) hashes the
// four keys with the SplitMix64 finaliser, so any pattern of any batch is
// reproducible on its own.  Pattern p: 8 Gaussian blobs (centre uniform in a
// centred disk of diameter n/4 by rejection, sigma U[2, 6] px, amplitude
// U[0.3, 1]), masked to the disk; I = |FFT(rho)|^2 scaled to `photons` and
// Poisson sampled (inversion for lambda < 10, Hoermann's transformed
// rejection PTRS above; both with bounded loops).  A negative photon count
// gives the noise-free expectation |FFT(rho)|^2 scaled to -photons.
#include <cuda_runtime.h>

#include <mutex>

#include <algorithm>
#include <cmath>
#include <string>

#include "cdx.h"
#include "cdx_host.h"
#include "cdx_types.h"
#include "cdx_unet.h"

namespace cdx {
namespace fm {

__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ unsigned long long key4(unsigned long long seed, unsigned long long pat,
                                                            unsigned long long stream, unsigned long long i) {
  unsigned long long h = mix64(seed + 0x9E3779B97F4A7C15ull);
  h = mix64(h ^ (pat * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull));
  h = mix64(h ^ (stream * 0xAEF17502108EF2D9ull + 0x4F1BBCDCBFA53E0Bull));
  return mix64(h ^ (i * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull));
}
// uniform in (0, 1), 53 bits
__host__ __device__ __forceinline__ double unif(unsigned long long seed, unsigned long long pat,
                                                unsigned long long stream, unsigned long long i) {
  return ((double)(key4(seed, pat, stream, i) >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}

enum { S_POS = 1, S_SIG = 2, S_AMP = 3, S_NOISE = 4 };
constexpr int kBlobs = 8;

// blob parameters (dx, dy, sigma, amplitude) of pattern `first + b`
__global__ void k_blob_params(int n, int count, unsigned long long seed, long long first, double* __restrict__ prm) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= count) return;
  const unsigned long long pat = (unsigned long long)(first + b);
  const double r = 0.25 * n / 2.0;
  for (int k = 0; k < kBlobs; ++k) {
    double dx = 0.0, dy = 0.0;
    for (int t = 0; t < 64; ++t) {   // acceptance pi/4 per try
      const double ux = unif(seed, pat, S_POS, (unsigned long long)(k * 128 + 2 * t));
      const double uy = unif(seed, pat, S_POS, (unsigned long long)(k * 128 + 2 * t + 1));
      const double x = (2.0 * ux - 1.0) * r, y = (2.0 * uy - 1.0) * r;
      if (x * x + y * y <= r * r) {
        dx = x;
        dy = y;
        break;
      }
    }
    double* q = prm + ((long long)b * kBlobs + k) * 4;
    q[0] = dx;
    q[1] = dy;
    q[2] = 2.0 + 4.0 * unif(seed, pat, S_SIG, (unsigned long long)k);
    q[3] = 0.3 + 0.7 * unif(seed, pat, S_AMP, (unsigned long long)k);
  }
}

// object (centred), its amplitude / phase / support targets
__global__ void k_blob_render(int n, long long total, const double* __restrict__ prm, float2* __restrict__ rho,
                              float* __restrict__ amp_t, float* __restrict__ ph_t, float* __restrict__ sup_t) {
  const long long P = (long long)n * n;
  const double c = n / 2.0, r = 0.25 * n / 2.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P;
    const int p = (int)(i - b * P);
    const int y = p / n, x = p - y * n;
    double v = 0.0;
    if ((y - c) * (y - c) + (x - c) * (x - c) <= r * r) {
      const double* q = prm + b * kBlobs * 4;
      for (int k = 0; k < kBlobs; ++k) {
        const double ey = y - c - q[4 * k], ex = x - c - q[4 * k + 1], s = q[4 * k + 2];
        v += q[4 * k + 3] * exp(-(ey * ey + ex * ex) / (2.0 * s * s));
      }
    }
    rho[i] = make_float2((float)v, 0.f);
    if (amp_t) amp_t[i] = (float)v;
    if (ph_t) ph_t[i] = 0.f;
    if (sup_t) sup_t[i] = v > 1e-3 ? 1.f : 0.f;
  }
}

// per-pattern sum of |F|^2 (fixed order)
__global__ void k_power_sum(const float2* __restrict__ F, long long P, double* __restrict__ sum) {
  __shared__ double r[256];
  const long long b = blockIdx.x;
  double s = 0.0;
  for (long long i = threadIdx.x; i < P; i += blockDim.x) {
    const float2 f = F[b * P + i];
    s += (double)f.x * f.x + (double)f.y * f.y;
  }
  r[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) r[threadIdx.x] += r[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) sum[b] = r[0];
}

__device__ double poisson_sample(double lam, unsigned long long seed, unsigned long long pat, unsigned long long px) {
  if (!(lam > 0.0)) return 0.0;
  unsigned long long ctr = px * 256ull;
  if (lam < 10.0) {
    const double L = exp(-lam);
    double prod = 1.0;
    for (int k = 0; k < 200; ++k) {
      prod *= unif(seed, pat, S_NOISE, ctr++);
      if (prod <= L) return (double)k;
    }
    return 200.0;
  }
  const double slam = sqrt(lam), loglam = log(lam);
  const double b = 0.931 + 2.53 * slam, a = -0.059 + 0.02483 * b;
  const double invalpha = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
  for (int t = 0; t < 64; ++t) {
    const double U = unif(seed, pat, S_NOISE, ctr++) - 0.5;
    const double V = unif(seed, pat, S_NOISE, ctr++);
    const double us = 0.5 - fabs(U);
    const double k = floor((2.0 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return k;
    if (k < 0.0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(invalpha) - log(a / (us * us) + b) <= -lam + k * loglam - lgamma(k + 1.0)) return k;
  }
  // not reached in practice (acceptance > 0.9 per try): normal approximation
  const double u1 = unif(seed, pat, S_NOISE, ctr++), u2 = unif(seed, pat, S_NOISE, ctr++);
  const double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  return fmax(0.0, floor(lam + slam * z + 0.5));
}

__global__ void k_intensity(const float2* __restrict__ F, const double* __restrict__ sum, int n, long long total,
                            double photons, unsigned long long seed, long long first, float* __restrict__ I) {
  const long long P = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / P;
    const float2 f = F[i];
    const double lam = ((double)f.x * f.x + (double)f.y * f.y) * (sum[b] > 0.0 ? fabs(photons) / sum[b] : 0.0);
    I[i] = photons > 0.0 ? (float)poisson_sample(lam, seed, (unsigned long long)(first + b), (unsigned long long)(i - b * P))
                         : (float)lam;
  }
}

// applyPoissonNoise_WO (src/gpu/cdi.cu:291-296) with scale = vars.scale =
// 1/exposure (init_cuda_image, cdi.cc:52): the pattern quantised to detector
// counts, plus zero-mean Poisson(noise_level) dark noise per pixel.
__global__ void k_ccd_noise(float* __restrict__ I, long long n, double noise_level, float scale, float rcolor,
                            unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double k = poisson_sample(noise_level, seed, 0x43434431ull, (unsigned long long)i);
    I[i] = scale * ((float)(int)(I[i] * rcolor / scale) + (float)k - (float)noise_level) / rcolor;
  }
}

// ccdRecord(data, wave, noiseLevel, state, exposure) on a float pattern (src/gpu/cdi.cu:260-266):
// k = Poisson(noiseLevel + rcolor I exposure), clamped below rcolor, I <- (k - noiseLevel) / rcolor,
// then times `post` (the caller's applyNorm)
__global__ void k_ccd_record(float* __restrict__ I, long long n, int noise_level, float exposure, int rcolor,
                             float post, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double lam = (double)((float)noise_level + (float)rcolor * I[i] * exposure);
    int k = (int)poisson_sample(lam > 0 ? lam : 0.0, seed, 0x43434452ull, (unsigned long long)i);
    if (k >= rcolor) k = rcolor - 1;
    I[i] = (float)(k - noise_level) / (float)rcolor * post;
  }
}

}  // namespace fm
}  // namespace cdx

using namespace cdx;
using namespace cdx::fm;

namespace {

// Scratch of cdx_forward_model (blob parameters, power sums, the complex
// field), kept per device and grown only when a call needs more, so that a
// training loop calling it every step allocates once.  `done` marks the end of
// the last call's use; a call on another stream waits for it on the device.
struct FmScratch {
  char* p = nullptr;
  size_t bytes = 0;
  cudaEvent_t done = nullptr;
};
std::mutex g_fm_mu;
FmScratch g_fm[64];

}  // namespace

extern "C" int cdx_forward_model(int n, int count, unsigned long long seed, long long first, double photons,
                                 float* intensity, float* amp_t, float* phase_t, float* support_t, void* stream) {
  if (!intensity || count < 1 || first < 0 || !(photons != 0.0) || photons != photons)
    return set_error(CDX_ERR_ARG, "bad forward-model argument");
  if (!cdx_size_supported(n)) return set_error(CDX_ERR_SIZE, "unsupported pattern size");
  cudaStream_t st = (cudaStream_t)stream;
  const long long P = (long long)n * n, tot = P * count;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_sum = al(sizeof(double) * count * kBlobs * 4);
  const size_t o_rho = o_sum + al(sizeof(double) * count);
  const size_t need = o_rho + sizeof(float2) * tot;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) return set_error(CDX_ERR_CUDA, "forward model: no usable device");
  std::lock_guard<std::mutex> lk(g_fm_mu);
  FmScratch& w = g_fm[dev];
  if (!w.done && (e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming)) != cudaSuccess)
    return set_error(CDX_ERR_CUDA, std::string("forward model event: ") + cudaGetErrorString(e));
  if (w.bytes < need) {
    if (w.p) {
      cudaEventSynchronize(w.done);
      cudaFree(w.p);
      w.p = nullptr;
      w.bytes = 0;
    }
    if ((e = cudaMalloc(&w.p, need)) != cudaSuccess) {
      w.p = nullptr;
      return set_error(CDX_ERR_NOMEM, std::string("forward model scratch: ") + cudaGetErrorString(e));
    }
    w.bytes = need;
  } else if ((e = cudaStreamWaitEvent(st, w.done, 0)) != cudaSuccess) {
    return set_error(CDX_ERR_CUDA, std::string("forward model wait: ") + cudaGetErrorString(e));
  }
  double* prm = (double*)w.p;
  double* sum = (double*)(w.p + o_sum);
  float2* rho = (float2*)(w.p + o_rho);
  k_blob_params<<<(count + 127) / 128, 128, 0, st>>>(n, count, seed, first, prm);
  const int g = (int)std::min<long long>((tot + 255) / 256, sm_count() * 32);
  k_blob_render<<<g, 256, 0, st>>>(n, tot, prm, rho, amp_t, phase_t, support_t);
  if ((e = cudaGetLastError()) != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("render: ") + cudaGetErrorString(e));
  int rc = cdx_fft2(rho, rho, n, n, count, 0, st);
  if (rc == CDX_OK) {
    k_power_sum<<<count, 256, 0, st>>>(rho, P, sum);
    k_intensity<<<g, 256, 0, st>>>(rho, sum, n, tot, photons, seed, first, intensity);
    if ((e = cudaGetLastError()) != cudaSuccess)
      rc = set_error(CDX_ERR_CUDA, std::string("intensity: ") + cudaGetErrorString(e));
  }
  cudaEventRecord(w.done, st);
  return rc;
}

extern "C" int cdx_ccd_noise(float* pattern, long long count, float noise_level, float exposure, int rcolor,
                             unsigned long long seed, void* stream) {
  if (!pattern || count < 0 || !(noise_level >= 0.f) || !(exposure > 0.f) || rcolor <= 0)
    return set_error(CDX_ERR_ARG, "bad CCD-noise argument");
  if (count == 0) return CDX_OK;
  const int g = (int)std::min<long long>((count + 255) / 256, sm_count() * 32);
  k_ccd_noise<<<g, 256, 0, (cudaStream_t)stream>>>(pattern, count, (double)noise_level, 1.f / exposure, (float)rcolor,
                                                    seed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("ccd noise: ") + cudaGetErrorString(e));
  return CDX_OK;
}

// multiplyFresnelPhase_Device (cudaConfig.cu:1095-1101): a <- a exp(i f ((x - rows/2)^2 + (y - cols/2)^2))
// on the entries that are not zero, the squared distance in integers and the phase in float
__global__ void k_fresnel_phase(float2* __restrict__ a, int rows, int cols, long long n, float f) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long k = i % ((long long)rows * cols);
    const int dx = (int)(k / cols) - (rows >> 1), dy = (int)(k % cols) - (cols >> 1);
    const float ph = f * (float)(dx * dx + dy * dy);
    float s, c;
    sincosf(ph, &s, &c);
    const float2 v = a[i];
    if (v.x != 0.f || v.y != 0.f) a[i] = make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

extern "C" float cdx_fresnel_factor(double lambda, double distance, double pixelsize, int rows, int remove) {
  // propagator members are float (propagator.hpp:9-13); pi lambda d / (pixelsize row)^2 in double
  const float lam = (float)lambda, dist = (float)distance, px = (float)pixelsize;
  const float side = px * (float)rows;
  const double f = M_PI * (double)lam * (double)dist / (double)(side * side);
  return (float)(remove ? -f : f);
}

extern "C" int cdx_fresnel_phase(void* field, int rows, int cols, int batch, float factor, void* stream) {
  if (!field || rows < 1 || cols < 1 || batch < 1) return set_error(CDX_ERR_ARG, "bad Fresnel-phase argument");
  const long long n = (long long)rows * cols * batch;
  const int g = (int)std::min<long long>((n + 255) / 256, sm_count() * 32);
  k_fresnel_phase<<<g, 256, 0, (cudaStream_t)stream>>>((float2*)field, rows, cols, n, factor);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("Fresnel phase: ") + cudaGetErrorString(e));
  return CDX_OK;
}

extern "C" int cdx_ccd_record(float* pattern, long long count, int noise_level, float exposure, int rcolor, float post,
                              unsigned long long seed, void* stream) {
  if (!pattern || count < 0 || noise_level < 0 || !(exposure > 0.f) || rcolor <= 0)
    return set_error(CDX_ERR_ARG, "bad CCD-record argument");
  if (count == 0) return CDX_OK;
  const int g = (int)std::min<long long>((count + 255) / 256, sm_count() * 32);
  k_ccd_record<<<g, 256, 0, (cudaStream_t)stream>>>(pattern, count, noise_level, exposure, rcolor, post, seed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("ccd record: ") + cudaGetErrorString(e));
  return CDX_OK;
}
