// C ABI of the ptychographic reconstruction (include/cdx_ptycho.h).
//
// A handle owns the object O and its momentum history, the probe P, its
// step accumulator, the pattern stack (column-tiled, so the column pass
// stages a pattern tile with 16-byte cp.async), the work array W and the
// device scalars of ptycho::iterate (util/ptycho.cpp:429-736).  Nothing in a
// sweep goes back to the host: the probe and object maxima, the scale
// balance, the far-field centroid and the momentum phase are reduced and
// consumed on the device, and the scan order and momentum coefficients of the
// whole run are uploaded before it.  One sweep (three kernels per scan
// position, plus the per-iteration steps) is captured once per phase into a
// CUDA graph and replayed; the kernels read the iteration from a device
// counter that the graph's last node advances.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cdx.h"
#include "../../include/cdx_ptycho.h"
#include "cdx_fft.cuh"
#include "cdx_host.h"
#include "cdx_ptycho.cuh"
#include "cdx_pty_zernike.cuh"
#include "cdx_types.h"

using namespace cdx;

#define PTY_CK(call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return set_error(CDX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
#define PTY_RET(call)              \
  do {                             \
    int r_ = (call);               \
    if (r_ != CDX_OK) return r_;   \
  } while (0)

namespace cdx {
int device_twiddles(int n, float2** out);   // cdx_api.cu: per-(device, length) table
#define CDX_PTY_EXTERN(N)                                                           \
  extern template cudaError_t pty_prepare<N>();                                     \
  extern template cudaError_t pty_launch_fwd<N>(const PtyArgs&, cudaStream_t);      \
  extern template cudaError_t pty_launch_upd<N>(const PtyArgs&, cudaStream_t);      \
  extern template cudaError_t pty_launch_col<N>(const PtyArgs&, cudaStream_t);
CDX_PTY_EXTERN(16) CDX_PTY_EXTERN(24) CDX_PTY_EXTERN(32) CDX_PTY_EXTERN(48) CDX_PTY_EXTERN(64)
CDX_PTY_EXTERN(96) CDX_PTY_EXTERN(128) CDX_PTY_EXTERN(192) CDX_PTY_EXTERN(256) CDX_PTY_EXTERN(384)
CDX_PTY_EXTERN(512) CDX_PTY_EXTERN(768) CDX_PTY_EXTERN(1024) CDX_PTY_EXTERN(1536) CDX_PTY_EXTERN(2048)
CDX_PTY_EXTERN(3072) CDX_PTY_EXTERN(4096)
}  // namespace cdx

namespace {

constexpr int kRedBlocks = 608;        // reduction CTAs (four per SM); the fused finalisers assume 256 threads
constexpr int kUpdateProbeIter = 400;  // util/ptycho.cpp:441
constexpr int kPositionUpdateIter = 500;   // util/ptycho.cpp:442
constexpr int kNoiseProjIter = 2000;       // applyMod instead of applyModAccurate (util/ptycho.cpp:536-545)
constexpr float kRcolor = 65535.f;         // rcolor (include/format.hpp:21)

typedef cudaError_t (*PtyPrep)();
typedef cudaError_t (*PtyLaunch)(const PtyArgs&, cudaStream_t);
struct PtyKernels {
  PtyPrep prep = nullptr;
  PtyLaunch fwd = nullptr, upd = nullptr, col = nullptr;
  int L = 0;
};
#define PTY_CASE(N) \
  case N: k.prep = &pty_prepare<N>; k.fwd = &pty_launch_fwd<N>; k.upd = &pty_launch_upd<N>; \
          k.col = &pty_launch_col<N>; k.L = Geom<N>::L; return true;
bool pty_kernels(int n, PtyKernels& k) {
  switch (n) {
    PTY_CASE(16) PTY_CASE(24) PTY_CASE(32) PTY_CASE(48) PTY_CASE(64) PTY_CASE(96) PTY_CASE(128)
    PTY_CASE(192) PTY_CASE(256) PTY_CASE(384) PTY_CASE(512) PTY_CASE(768) PTY_CASE(1024)
    PTY_CASE(1536) PTY_CASE(2048) PTY_CASE(3072) PTY_CASE(4096)
    default: return false;
  }
}

// Device scalars of a sweep.  pmax/omax first: the update kernel reads them as scal[0], scal[1].
struct PtyScal {
  float pmax, omax;      // max |P|^2; object maximum (probe phase: both the balanced value)
  float thr, sf, isf;    // applyThreshold level, object scale, probe scale
  float shx, shy;        // far-field recentring shift (multiplyShift arguments)
  float phx, phy;        // unit phase of the object sum (multiplyConj by it)
  unsigned maxb[2];      // max reductions as float bits (non-negative values)
};

inline unsigned grid1(long long n, int t = 256) {
  long long b = (n + t - 1) / t;
  return (unsigned)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

// ------------------------------------------------------------------ kernels
// util/ptycho.cpp:485-509: the probe maximum; from iteration 400 the object
// maximum over the covered area, its threshold, the scale balance
// sf = (max|P|^2 / objMax)^(1/4) and the balanced maxima sqrt(objMax max|P|^2).
__device__ void pty_balance(PtyScal* s, int probe_phase) {
  const float pm = __uint_as_float(atomicAdd(&s->maxb[0], 0u));
  s->pmax = pm;
  if (!probe_phase) return;
  const float om = __uint_as_float(atomicAdd(&s->maxb[1], 0u));
  s->thr = sqrtf(om);
  const float sf = (float)pow((double)(pm / om), 0.25);
  s->sf = sf;
  s->isf = (float)(1.0 / (double)sf);
  const float m = sqrtf(om * pm);
  s->pmax = m;
  s->omax = m;
}

// True in one thread of the CTA that finishes last (the others' results are
// then visible); that thread resets the counter for the next launch.
__device__ __forceinline__ bool pty_last_block(unsigned* count) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(count, 1u) == gridDim.x - 1;
    if (last) *count = 0;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// max |x|^2 (times the mask) as float bits by atomic max; the CTA that
// finishes last computes the balance (balance < 0: none)
__global__ void k_pty_max_mod2(const float2* __restrict__ x, const float* __restrict__ mask, long long n,
                               unsigned* out, PtyScal* s, unsigned* count, int balance) {
  float m = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[i];
    float q = v.x * v.x + v.y * v.y;   // getMod2
    if (mask) q = q * mask[i];         // multiply(maxCache, maxCache, masksum)
    m = fmaxf(m, q);
  }
  for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
  if (balance < 0) return;
  if (pty_last_block(count) && threadIdx.x == 0) pty_balance(s, balance);
}

// applyThreshold(O, O, sqrt(objMax)) (src/gpu/cudaConfig.cu:397-406), then applyNorm by sf of O and its history.
__global__ void k_pty_obj_balance(float2* __restrict__ O, float2* __restrict__ Op, long long n, const PtyScal* s) {
  const float thr = s->thr, sf = s->sf;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 d = O[i];
    const float m2 = d.x * d.x + d.y * d.y;
    if (m2 > thr) {
      const float f = sqrtf(thr / m2);
      d.x = f * d.x;
      d.y = f * d.y;
    }
    d.x *= sf;
    d.y *= sf;
    O[i] = d;
    float2 q = Op[i];
    q.x *= sf;
    q.y *= sf;
    Op[i] = q;
  }
}

// applyNorm(pupilpatternWave, 1/sf) and applyNorm(probe_prev, 1/sf) (util/ptycho.cpp:506-507)
__global__ void k_pty_scale(float2* __restrict__ x, float2* __restrict__ y, long long n, const float* f) {
  const float s = *f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 v = x[i], w = y[i];
    v.x *= s;
    v.y *= s;
    w.x *= s;
    w.y *= s;
    x[i] = v;
    y[i] = w;
  }
}

// add(P, probeStep) then applyNorm(probeStep, 0) (util/ptycho.cpp:563-566)
__global__ void k_pty_add_step(float2* __restrict__ P, float2* __restrict__ st, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 p = P[i], s = st[i];
    p.x += s.x;
    p.y += s.y;
    P[i] = p;
    s.x *= 0.f;
    s.y *= 0.f;
    st[i] = s;
  }
}

// The middle of angularSpectrumPropagate(Reverse) (src/post_gpu/propagator.cc:31-49):
// applyNorm(1/(rows cols)), then multiplyPropagatePhase (src/gpu/cudaConfig.cu:669-679)
// between the two cudaConvertFO, i.e. at the signed frequency of each FFT-order element.
__global__ void k_pty_as_phase(float2* __restrict__ F, int rows, int cols, float inv_n, float a, float b) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols), y = (int)(i % cols);
    const int fx = x < rows / 2 ? x : x - rows;   // centred index minus rows/2
    const int fy = y < cols / 2 ? y : y - cols;
    float2 v = F[i];
    v.x *= inv_n;
    v.y *= inv_n;
    // phase = a sqrt(1 - q b) with a ~ 2 pi distance/lambda (1e4 rad and more): one
    // ulp of the root moves the phase by ~1e-3 rad, so the product and the
    // difference are rounded separately (no FMA contraction), as the host-built
    // reference evaluates them
    const float square = __fsub_rn(1.f, __fmul_rn((float)(fx * fx + fy * fy), b));
    if (square < 0) {
      F[i] = make_float2(0.f, 0.f);
      continue;
    }
    const float phase = __fmul_rn(a, sqrtf(square));
    float sn, cs;
    sincosf(phase, &sn, &cs);
    F[i] = cmul(v, make_float2(cs, sn));
  }
}

// crop to the centred pd x pd square, applyMask with the disk
// createCircleMask(pupilSupport, (pd+1)/2, (pd+1)/2, pd/2) (int centre), pad back
// (util/ptycho.cpp:610-623).
__global__ void k_pty_pupil_mask(float2* __restrict__ P, int rows, int cols, int pd) {
  const long long n = (long long)rows * cols;
  const int r0 = (rows - pd) / 2, c0 = (cols - pd) / 2;
  const int x0 = (int)((float)(pd + 1) / 2), y0 = x0;
  const float r = (float)pd / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols) - r0, y = (int)(i % cols) - c0;
    bool keep = x >= 0 && x < pd && y >= 0 && y < pd;
    if (keep) {
      const float dx = (float)(x - x0), dy = (float)(y - y0);
      keep = sqrtf(dx * dx + dy * dy) < r;
    }
    if (!keep) P[i] = make_float2(0.f, 0.f);
  }
}

// findMiddle of |cudaConvertFO(FFT(P))|^2 (src/post_gpu/misc.cc:27-42): per-CTA sums of
// m, m ((x + 0.5)/rows - 0.5), m ((y + 0.5)/cols - 0.5) at the centred coordinates.
__global__ void k_pty_far_part(const float2* __restrict__ F, int rows, int cols, double* part, PtyScal* s,
                               unsigned* count) {
  __shared__ double red[3][8];
  const long long n = (long long)rows * cols;
  double s0 = 0, s1 = 0, s2 = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols), y = (int)(i % cols);
    const int xc = (x + rows / 2) % rows, yc = (y + cols / 2) % cols;
    const float2 v = F[i];
    const float m = v.x * v.x + v.y * v.y;
    s0 += m;
    s1 += (float)(m * ((xc + 0.5) / rows - 0.5));
    s2 += (float)(m * ((yc + 0.5) / cols - 0.5));
  }
  for (int o = 16; o; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = s0; red[1][w] = s1; red[2][w] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0, t1 = 0, t2 = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { t0 += red[0][k]; t1 += red[1][k]; t2 += red[2][k]; }
    part[3 * blockIdx.x] = t0;
    part[3 * blockIdx.x + 1] = t1;
    part[3 * blockIdx.x + 2] = t2;
  }
  // the CTA that finishes last sums the partials in index order:
  // middle = (sum_x / sum, sum_y / sum) in float; multiplyShift(P, mid.x rows - 0.5, mid.y cols - 0.5)
  if (!pty_last_block(count)) return;
  __shared__ double fin[8];
  double t0 = 0, t1 = 0, t2 = 0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    t0 += __ldcg(part + 3 * k);
    t1 += __ldcg(part + 3 * k + 1);
    t2 += __ldcg(part + 3 * k + 2);
  }
  t0 = block_sum_d<256>(t0, fin);
  t1 = block_sum_d<256>(t1, fin);
  t2 = block_sum_d<256>(t2, fin);
  if (threadIdx.x == 0) {
    const float mx = (float)t1 / (float)t0, my = (float)t2 / (float)t0;
    s->shx = (float)((double)(mx * rows) - 0.5);
    s->shy = (float)((double)(my * cols) - 0.5);
  }
}
// multiplyShift (src/gpu/cudaConfig.cu:373-378)
__global__ void k_pty_mshift(float2* __restrict__ P, int rows, int cols, const PtyScal* s) {
  const float sx = s->shx, sy = s->shy;
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols), y = (int)(i % cols);
    const float t = sx * (x - rows / 2) / rows + sy * (y - cols / 2) / cols;
    const float ph = (float)(-2 * M_PI * (double)t);
    float sn, cs;
    sincosf(ph, &sn, &cs);
    P[i] = cmul(P[i], make_float2(cs, sn));
  }
}

// findSum of O (times the overlap mask for the momentum step): float sums per
// thread (the reference's CUB sum is float), double across threads and CTAs in
// a fixed order; the CTA that finishes last forms the unit phase:
// sum /= |sum| with cabs in double for the momentum step (util/ptycho.cpp:672-673),
// with the float hypot for the final phase removal (733)
__global__ void k_pty_csum(const float2* __restrict__ O, const float* __restrict__ m, long long n, double* part,
                           PtyScal* s, unsigned* count, int final_phase) {
  __shared__ double red[2][8];
  float ax = 0.f, ay = 0.f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 v = O[i];
    if (m) { const float f = m[i]; v.x *= f; v.y *= f; }
    ax += v.x;
    ay += v.y;
  }
  double sx = ax, sy = ay;
  for (int o = 16; o; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = sx; red[1][w] = sy; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) { a += red[0][k]; b += red[1][k]; }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
  if (!pty_last_block(count)) return;
  __shared__ double fin[8];
  double a = 0, b = 0;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
    a += __ldcg(part + 2 * k);
    b += __ldcg(part + 2 * k + 1);
  }
  a = block_sum_d<256>(a, fin);
  b = block_sum_d<256>(b, fin);
  if (threadIdx.x != 0) return;
  const float re = (float)a, im = (float)b;
  if (final_phase) {
    const float h = hypotf(re, im);
    s->phx = re / h;
    s->phy = im / h;
  } else {
    const double h = hypot((double)re, (double)im);
    s->phx = (float)(re / h);
    s->phy = (float)(im / h);
  }
}
// The momentum step (util/ptycho.cpp:669-681): both iterates times conj(phase),
// O_prev <- O - O_prev, then O_prev <- O + c O_prev, and the two swap.
__global__ void k_pty_momentum(float2* __restrict__ O, float2* __restrict__ Op, long long n, const PtyScal* s,
                               const float* coef, const int* iter) {
  const float2 ph = make_float2(s->phx, -s->phy);
  const float c = coef[*iter];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 o = cmul(O[i], ph);
    const float2 p = cmul(Op[i], ph);
    float2 d;
    d.x = o.x + p.x * -1.f;
    d.y = o.y + p.y * -1.f;
    float2 e;
    e.x = o.x + d.x * c;
    e.y = o.y + d.y * c;
    O[i] = e;
    Op[i] = o;
  }
}
__global__ void k_pty_conj_phase(float2* __restrict__ O, long long n, const PtyScal* s) {
  const float2 ph = make_float2(s->phx, -s->phy);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    O[i] = cmul(O[i], ph);
}
__global__ void k_pty_next(int* iter) { *iter += 1; }

// ------------------------------------------------------------ scan-position refinement
// (positionUncertainty > 0: every 20 sweeps from 500, util/ptycho.cpp:511-585)

// getWindow of the position visited k-th (zero outside the object), row-major rows x cols
__global__ void k_pty_pos_window(const float2* __restrict__ O, int obj_rows, int obj_cols, const int2* __restrict__ win,
                                 const int* order, const int* iter, int nscan, int k, float2* __restrict__ gw,
                                 int rows, int cols) {
  const int2 w = win[order[*iter * nscan + k]];
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int ox = w.x + (int)(i / cols), oy = w.y + (int)(i % cols);
    gw[i] = ox >= 0 && ox < obj_rows && oy >= 0 && oy < obj_cols ? O[(long long)ox * obj_cols + oy] : make_float2(0.f, 0.f);
  }
}

// updatePosition's spectral derivatives (util/ptycho.cpp:366-371): the window's spectrum
// (FFT order) centred and scaled by s1 = sqrt(1/n), times (x/rows - 0.5) (frame D) and
// (y/cols - 0.5) (frame D + n) at the centred coordinates, back to FFT order times 1/n
__global__ void k_pty_pos_deriv(float2* __restrict__ D, int rows, int cols, float s1, float nrm) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const int xc = (r + (rows >> 1)) % rows, yc = (c + (cols >> 1)) % cols;
    const float sx = (float)xc * (1.0f / (float)rows) - 0.5f, sy = (float)yc * (1.0f / (float)cols) - 0.5f;
    float2 v = D[i];
    v.x *= s1;
    v.y *= s1;
    D[i] = make_float2(v.x * sx * nrm, v.y * sx * nrm);
    D[i + n] = make_float2(v.x * sy * nrm, v.y * sy * nrm);
  }
}

// multiply(cache, cache, probe) on both frames
__global__ void k_pty_pos_probe(float2* __restrict__ D, const float2* __restrict__ P, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 p = P[i];
    D[i] = cmul(D[i], p);
    D[i + n] = cmul(D[i + n], p);
  }
}

// calcPartial (src/gpu/ptycho.cu:156-169) on both frames against Fn * norm, summed (findSum):
// (Fn.x d.y - Fn.y d.x)(1 - sqrt(max(I + 1e-3, 0) / (|Fn|^2 + 1e-3))); beamstop pixels add
// nothing.  Per-CTA double sums, the last CTA writes grad[si] and grad[si + nscan].
__global__ void k_pty_pos_partial(const float2* __restrict__ Fn, const float2* __restrict__ D, const float* __restrict__ pats,
                                  long long pat_stride, const float* __restrict__ bs, int rows, int cols, int tl, float norm,
                                  const int* order, const int* iter, int nscan, int k, double* part, unsigned* count,
                                  float* grad) {
  __shared__ double red[2][8];
  const int si = order[*iter * nscan + k];
  const float* pat = pats + (long long)si * pat_stride;
  const long long n = (long long)rows * cols;
  double ax = 0, ay = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const long long ti = pty_tiled(r, c, rows, tl);
    if (bs && bs[ti] > 0.5f) continue;
    float2 f = Fn[i];
    f.x *= norm;
    f.y *= norm;
    const float fm2 = f.x * f.x + f.y * f.y;
    float fact = pat[ti] + 1e-3f;
    if (fact < 0.f) fact = 0.f;
    const float kf = 1.f - sqrtf(fact / (fm2 + 1e-3f));
    const float2 dx = D[i], dy = D[i + n];
    ax += (double)((f.x * dx.y - f.y * dx.x) * kf);
    ay += (double)((f.x * dy.y - f.y * dy.x) * kf);
  }
  for (int o = 16; o; o >>= 1) {
    ax += __shfl_xor_sync(0xffffffffu, ax, o);
    ay += __shfl_xor_sync(0xffffffffu, ay, o);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = ax; red[1][w] = ay; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { a += red[0][q]; b += red[1][q]; }
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
  if (!pty_last_block(count)) return;
  __shared__ double fin[8];
  double a = 0, b = 0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
    a += __ldcg(part + 2 * q);
    b += __ldcg(part + 2 * q + 1);
  }
  a = block_sum_d<256>(a, fin);
  b = block_sum_d<256>(b, fin);
  if (threadIdx.x != 0) return;
  grad[si] = (float)a;
  grad[si + nscan] = (float)b;
}

// addProbability(d_shifts, d_shift, 0.3, positionUncertainty) (cudaConfig.cu:808-817), the
// mean shift removed from every position (util/ptycho.cpp:569-577), the window origins
// round(scanpos + shift) renewed; mean[0..1] receives the mean shift.  One thread.
__global__ void k_pty_pos_update(float* __restrict__ shifts, const float* __restrict__ grad,
                                 const float* __restrict__ scanpos, int2* __restrict__ win, int nscan, float sigma,
                                 float* __restrict__ mean) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int j = 0; j < 2 * nscan; ++j) {
    const float d = shifts[j], v = grad[j] * 0.3f, t = d + v;
    if (fabsf(t) > fabsf(d)) {
      const float g = expf(-(t * t) / 2 / (sigma * sigma));   // gaussian(t, 0, sigma), cudaConfig.cu:24-26
      shifts[j] = d + v * g;
    } else {
      shifts[j] = t;
    }
  }
  for (int a = 0; a < 2; ++a) {
    double sum = 0;
    for (int i = 0; i < nscan; ++i) sum += shifts[a * nscan + i];
    const float m = (float)sum / (float)nscan;
    mean[a] = m;
    for (int i = 0; i < nscan; ++i) shifts[a * nscan + i] = shifts[a * nscan + i] - m;
  }
  for (int i = 0; i < nscan; ++i)
    win[i] = make_int2((int)roundf(scanpos[i] + shifts[i]), (int)roundf(scanpos[nscan + i] + shifts[nscan + i]));
}

// shiftWave(objFFT, wave, -mean) between its transforms (src/post_gpu/misc.cc:106-113): the
// spectrum (FFT order) times multiplyShift's phase at the centred coordinates and 1/(rows cols)
__global__ void k_pty_pos_oshift(float2* __restrict__ S, int rows, int cols, const float* __restrict__ mean) {
  const float shx = -mean[0], shy = -mean[1], inv = (float)(1. / ((double)rows * cols));
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const int x = (r + (rows >> 1)) % rows, y = (c + (cols >> 1)) % cols;
    const float t = shx * (float)(x - rows / 2) / (float)rows + shy * (float)(y - cols / 2) / (float)cols;
    float sn, cs;
    sincosf((float)(-2 * M_PI * (double)t), &sn, &cs);
    float2 v = cmul(S[i], make_float2(cs, sn));
    v.x *= inv;
    v.y *= inv;
    S[i] = v;
  }
}

// FISTA_step (src/post_gpu/FISTA.cc:109-135) of the object, one TV proximal step,
// fused: o = b * s (s = 0.125/lambda), forward differences p (rows) and q
// (columns) of o, each component of (p, q) scaled to modulus <= 1 (diffMax),
// lpq = p + q - p(x-1) - q(y-1) (calcLpq, no wrap), out = b - lambda lpq
// (src/gpu/cudaConfig.cu:1124-1188).
__device__ __forceinline__ void pty_tv_pq(const float2* __restrict__ b, int rows, int cols, int x, int y, float s,
                                          float2& p, float2& q) {
  const long long i = (long long)x * cols + y;
  const float2 o = make_float2(b[i].x * s, b[i].y * s);
  p = o;
  q = o;
  if (x != rows - 1) {
    const float2 d = b[i + cols];
    p = make_float2(o.x - d.x * s, o.y - d.y * s);
  }
  if (y != cols - 1) {
    const float2 d = b[i + 1];
    q = make_float2(o.x - d.x * s, o.y - d.y * s);
  }
  float m = hypotf(p.x, q.x);
  if (m > 1) { p.x /= m; q.x /= m; }
  m = hypotf(p.y, q.y);
  if (m > 1) { p.y /= m; q.y /= m; }
}
__global__ void k_pty_fista(const float2* __restrict__ b, float2* __restrict__ out, int rows, int cols, float s,
                            float lam) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols), y = (int)(i % cols);
    float2 p, q, l;
    pty_tv_pq(b, rows, cols, x, y, s, p, q);
    l = make_float2(p.x + q.x, p.y + q.y);
    if (x >= 1) {
      float2 pm, qm;
      pty_tv_pq(b, rows, cols, x - 1, y, s, pm, qm);
      l.x -= pm.x;
      l.y -= pm.y;
    }
    if (y >= 1) {
      float2 pn, qn;
      pty_tv_pq(b, rows, cols, x, y - 1, s, pn, qn);
      l.x -= qn.x;
      l.y -= qn.y;
    }
    const float2 v = b[i];
    out[i] = make_float2(v.x + l.x * -lam, v.y + l.y * -lam);
  }
}

// the probe's momentum step on the Zernike sweeps (util/ptycho.cpp:682-686):
// P_prev <- P - P_prev, then P_prev <- P + c P_prev, and the two swap
__global__ void k_pty_probe_momentum(float2* __restrict__ P, float2* __restrict__ Pp, long long n, const float* coefz,
                                     const int* iter) {
  const float c = coefz[*iter];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 p = P[i], q = Pp[i];
    float2 d;
    d.x = p.x + q.x * -1.f;
    d.y = p.y + q.y * -1.f;
    P[i] = make_float2(p.x + d.x * c, p.y + d.y * c);
    Pp[i] = p;
  }
}

// Overlap mask (util/ptycho.cpp:470-479): the disk createCircleMask(row>>1, column>>1,
// pupilSize/2) added at every truncated scan position (addWindow), then bitMap(> 0.5).
// The sums are small integers, so the atomic order does not matter.
__global__ void k_pty_masksum(float* __restrict__ msum, const int2* __restrict__ trunc_pos, int nscan, int rows, int cols,
                              int orow, int ocol, float radius) {
  const long long n = (long long)rows * cols * nscan;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(g / ((long long)rows * cols));
    const long long i = g - (long long)s * rows * cols;
    const int x = (int)(i / cols), y = (int)(i % cols);
    const float dx = (float)(x - (rows >> 1)), dy = (float)(y - (cols >> 1));
    if (!(sqrtf(dx * dx + dy * dy) < radius)) continue;
    const int ox = x + trunc_pos[s].x, oy = y + trunc_pos[s].y;
    if (ox < 0 || ox >= orow || oy < 0 || oy >= ocol) continue;
    atomicAdd(msum + (long long)ox * ocol + oy, 1.f);
  }
}
__global__ void k_pty_bitmap(float* __restrict__ m, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    m[i] = m[i] > 0.5f ? 1.f : 0.f;
}

// row-major <-> column-tiled (width 2^tl) of one rows x cols float array
__global__ void k_pty_tile(const float* __restrict__ in, float* __restrict__ out, int rows, int cols, int tl, int dir) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const long long t = pty_tiled(r, c, rows, tl);
    if (dir == 0) out[t] = in[i];
    else out[i] = in[t];
  }
}

// pupilFunc (src/gpu/ptycho.cu:123-130)
__global__ void k_pty_pupil_func(float2* __restrict__ P, int rows, int cols, float ps) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int sx = (int)(i / cols) - rows / 2, sy = (int)(i % cols) - cols / 2;
    P[i] = make_float2((sx * sx + sy * sy > (ps * ps) / 4) ? 0.f : 1.f, 0.f);
  }
}

// random (src/gpu/ptycho.cu:114-117): unit modulus, phase 2 pi u; u from a counter-based
// hash of (seed, pixel) (SplitMix64 finaliser) instead of curand MRG32k3a.
__device__ __forceinline__ unsigned long long pty_mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
__global__ void k_pty_random(float2* __restrict__ O, long long n, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = pty_mix64(seed * 0x9e3779b97f4a7c15ULL + (unsigned long long)i + 1);
    const float u = (float)((h >> 40) + 1) * (1.0f / 16777216.0f);
    float s, c;
    sincosf((float)(u * 2 * M_PI), &s, &c);
    O[i] = make_float2(c, s);
  }
}

// createPattern's getMod2(pattern, esw, 1/(rows cols)), applyNorm(exposure),
// applyNorm(1/exposure) (util/ptycho.cpp:336-358), stored column-tiled
// (with useBS, applySupport(pattern, beamstop) zeroes the stopped pixels; with simCCDbit the
// exposure scalings are left to the detector model that follows)
__global__ void k_pty_sim_mod2(const float2* __restrict__ F, float* __restrict__ out, int rows, int cols, int tl,
                               float inv_n, float expo, float inv_expo, const float* __restrict__ bs, int ccd) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 v = F[i];
    const long long ti = pty_tiled((int)(i / cols), (int)(i % cols), rows, tl);
    float m = (v.x * v.x + v.y * v.y) * inv_n;
    if (bs && bs[ti] > 0.f) m = 0.f;
    if (!ccd) {
      m *= expo;
      m *= inv_expo;
    }
    out[ti] = m;
  }
}

// createBeamStop (src/post_gpu/misc.cc:191-195): createCircleMask(row>>1, column>>1,
// beamStopSize, isFreq = 1), stored column-tiled
__global__ void k_pty_beamstop(float* __restrict__ bs, int rows, int cols, int tl, float r) {
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    int x = (int)(i / cols), y = (int)(i % cols);
    const int xi = x, yi = y;
    x = x >= rows / 2 ? x - rows / 2 : x + rows / 2;
    y = y >= cols / 2 ? y - cols / 2 : y + cols / 2;
    const float dx = (float)(x - (rows >> 1)), dy = (float)(y - (cols >> 1));
    bs[pty_tiled(xi, yi, rows, tl)] = sqrtf(dx * dx + dy * dy) < r ? 1.f : 0.f;
  }
}

// ----------------------------------------------------------- host helpers
// The C library's rand() (TYPE_3 additive feedback generator of degree 31,
// separation 3, seeded through the Park-Miller minimal standard), restated so
// the scan orders do not depend on the process's rand() state.
struct LibcRand {
  std::vector<int32_t> r;
  size_t k = 0;
  explicit LibcRand(unsigned seed) {
    r.resize(344);
    r[0] = (int32_t)(seed == 0 ? 1 : seed);
    for (int i = 1; i < 31; ++i) {
      const int64_t hi = r[i - 1] / 127773, lo = r[i - 1] % 127773;
      int64_t w = 16807 * lo - 2836 * hi;
      if (w < 0) w += 2147483647;
      r[i] = (int32_t)w;
    }
    for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
    for (int i = 34; i < 344; ++i) r[i] = (int32_t)((uint32_t)r[i - 31] + (uint32_t)r[i - 3]);
    k = 344;
  }
  int next() {
    const int32_t v = (int32_t)((uint32_t)r[k - 31] + (uint32_t)r[k - 3]);
    r.push_back(v);
    ++k;
    return (int)((uint32_t)v >> 1);
  }
};

void scan_orders_host(int nscan, int n_iter, unsigned seed, int* out) {
  LibcRand g(seed);
  std::vector<int> order(nscan);
  for (int i = 0; i < nscan; ++i) order[i] = i;
  for (int it = 0; it < n_iter; ++it) {
    for (int i = nscan - 1; i > 0; --i) {   // shuffle_array (util/ptycho.cpp:28-38)
      const int j = g.next() % (i + 1);
      std::swap(order[i], order[j]);
    }
    std::memcpy(out + (size_t)it * nscan, order.data(), sizeof(int) * nscan);
  }
}

int ilog2(int v) {
  int l = 0;
  while ((1 << l) < v) ++l;
  return l;
}

}  // namespace

struct cdx_pty {
  cdx_pty_params p{};
  cudaStream_t st = nullptr;
  bool own_st = false;
  PtyKernels kr, kc;     // column pass (length rows), row passes (length cols)
  float2* tw_r = nullptr;
  float2* tw_c = nullptr;
  int tl = 0;            // log2 of the column pass's tile width
  long long npx = 0, onpx = 0, pat_stride = 0;
  float2 *O = nullptr, *Op = nullptr, *P = nullptr, *step = nullptr, *W = nullptr, *tmp = nullptr, *pupil = nullptr;
  float *pats = nullptr, *bs = nullptr, *msum = nullptr, *coef = nullptr;
  int2 *win = nullptr, *tpos = nullptr;
  int *order = nullptr, *iter = nullptr;
  PtyScal* scal = nullptr;
  double* part = nullptr;
  unsigned* cnt = nullptr;   // last-CTA tickets of the fused reductions (reset by their last CTA)
  int* derr = nullptr;       // bulk staging timeouts of the column kernel (bit 0)
  int order_cap = 0, coef_cap = 0;
  bool have_scan = false, have_pats = false, have_obj = false, have_probe = false;
  // one sweep per kind: phase (object, probe, probe + noise projection) x FISTA x probe momentum
  // x Zernike pupil fit
  // x position refinement
  cudaGraphExec_t graph[48] = {};
  float2* Pp = nullptr;       // probe momentum history (Zernike sweeps)
  float2* fista = nullptr;    // FISTA output before it replaces the object
  float* coefz = nullptr;     // probe momentum coefficients per sweep
  float4* zk_tab = nullptr;   // Zernike fit: pixel table of the pupil crop
  float2* zk_part = nullptr;  // Zernike fit: partial coefficients per projection CTA
  float2* zk_coef = nullptr;  // Zernike fit: the thresholded coefficients
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float last_ms = 0.f;
  float lam = 0, dist = 0, res = 0;   // propagate_pupil members (float)
  float fresnel = 0.f;                // propagate_esw's Fresnel phase factor (isFresnel), else 0
  // scan-position refinement (position_uncertainty > 0)
  float *shifts = nullptr, *grad = nullptr, *scanpos = nullptr, *pmean = nullptr;
  float2 *fn = nullptr, *gw = nullptr, *dxy = nullptr, *dtmp = nullptr, *otmp = nullptr;
  float2 *tw_or = nullptr, *tw_oc = nullptr;   // object-size twiddles (rows, cols)
  RowLaunch orow = nullptr;                    // object row pass (length obj_cols)
  ColLaunch ocol = nullptr;                    // object column pass (length obj_rows)
  std::vector<int2> win0;                      // nominal window origins
};

namespace {

// unnormalised 2-D FFT of `batch` row-major rows x cols frames, in -> out
int fft2g(cudaStream_t st, const float2* in, float2* out, bool inv, int rows, int cols, const float2* twr,
          const float2* twc, RowLaunch rl, ColLaunch cl, int batch) {
  RowArgs r{};
  r.in = in;
  r.out = out;
  r.in_stride = r.out_stride = (long long)rows * cols;
  r.tw = twc;
  r.rows = rows;
  r.mode = ROW_FFT;
  r.inv = inv;
  r.scale = 1.f;
  PTY_CK(rl(r, batch, st));
  ColArgs c{};
  c.in = out;
  c.out = out;
  c.in_stride = c.out_stride = (long long)rows * cols;
  c.tw = twr;
  c.cols = cols;
  c.mode = COL_FFT;
  c.inv = inv;
  c.scale = 1.f;
  PTY_CK(cl(c, batch, st));
  return CDX_OK;
}

int fft2(cdx_pty* t, const float2* in, float2* out, bool inv, int batch = 1) {
  return fft2g(t->st, in, out, inv, t->p.rows, t->p.cols, t->tw_r, t->tw_c, row_launcher(t->p.cols),
               col_launcher(t->p.rows), batch);
}

// propagator::angularSpectrumPropagate(Reverse) of P in place (src/post_gpu/propagator.cc:31-49),
// the propagator's lambda, distance and pixel size being float members.
int angular_spectrum(cdx_pty* t, float2* P, bool reverse) {
  const int R = t->p.rows, C = t->p.cols;
  float a, b;
  if (!reverse) {
    const float loi = t->lam / (t->res * R);
    a = (float)(2 * M_PI * (double)t->dist / (double)t->lam);
    b = loi * loi;
  } else {
    const float iol = t->res * R / t->lam;
    a = (float)(-2 * M_PI * (double)t->dist / (double)t->lam);
    b = (float)(1. / (double)(iol * iol));
  }
  PTY_RET(fft2(t, P, t->tmp, false));
  k_pty_as_phase<<<grid1(t->npx), 256, 0, t->st>>>(t->tmp, R, C, (float)(1. / ((double)R * C)), a, b);
  PTY_CK(cudaGetLastError());
  return fft2(t, t->tmp, P, true);
}

PtyArgs pass_args(cdx_pty* t, int k, bool probe_phase, bool noise_proj = false) {
  PtyArgs a{};
  a.W = t->W;
  a.obj = t->O;
  a.probe = t->P;
  a.step = t->step;
  a.pats = t->pats;
  a.bs = t->p.use_bs ? t->bs : nullptr;
  a.order = t->order;
  a.iter = t->iter;
  a.win = t->win;
  a.scal = &t->scal->pmax;
  a.pat_stride = t->pat_stride;
  a.rows = t->p.rows;
  a.cols = t->p.cols;
  a.obj_rows = t->p.obj_rows;
  a.obj_cols = t->p.obj_cols;
  a.tl = t->tl;
  a.k = k;
  a.nscan = t->p.nscan;
  a.probe_phase = probe_phase;
  a.norm = (float)(1. / std::sqrt((double)t->p.rows * t->p.cols));
  a.maximum = (float)(1. / t->p.exposure) * 0.95f;
  a.obj_step = probe_phase ? 0.5f : 1.f;
  a.pss = (float)(1. / t->p.nscan);
  a.noise_proj = noise_proj;
  a.noise_level = t->p.noise_level;
  a.ccd_scale = (float)(1. / t->p.exposure);
  a.rcolor = kRcolor;
  a.err = t->derr;
  a.fresnel = t->fresnel;
  return a;
}

// One sweep of ptycho::iterate (util/ptycho.cpp:484-690) for the iteration the device counter names.
int enqueue_sweep(cdx_pty* t, bool probe_phase, bool noise_proj, bool fista, bool probe_momentum, bool zernike,
                  bool posupd) {
  cudaStream_t st = t->st;
  const long long n = t->npx, on = t->onpx;
  PTY_CK(cudaMemsetAsync(t->scal->maxb, 0, sizeof(t->scal->maxb), st));
  k_pty_max_mod2<<<grid1(n), 256, 0, st>>>(t->P, nullptr, n, &t->scal->maxb[0], t->scal, t->cnt,
                                            probe_phase ? -1 : 0);
  if (probe_phase)
    k_pty_max_mod2<<<grid1(on), 256, 0, st>>>(t->O, t->msum, on, &t->scal->maxb[1], t->scal, t->cnt + 1, 1);
  if (probe_phase) {
    k_pty_obj_balance<<<grid1(on), 256, 0, st>>>(t->O, t->Op, on, t->scal);
    k_pty_scale<<<grid1(n), 256, 0, st>>>(t->P, t->Pp, n, &t->scal->isf);
  }
  PTY_CK(cudaGetLastError());
  const int rows = t->p.rows, cols = t->p.cols, ns = t->p.nscan;
  for (int k = 0; k < ns; ++k) {
    PtyArgs a = pass_args(t, k, probe_phase, noise_proj);
    a.tw = t->tw_c;
    PTY_CK(t->kc.fwd(a, st));
    if (posupd) {   // updatePosition (util/ptycho.cpp:360-385) before the projection
      ColArgs c{};   // Fn: the column FFT of W, row-major
      c.in = t->W;
      c.out = t->fn;
      c.in_tiled = 1;
      c.in_stride = t->pat_stride;
      c.out_stride = n;
      c.tw = t->tw_r;
      c.cols = cols;
      c.mode = COL_FFT;
      c.scale = 1.f;
      PTY_CK(col_launcher(rows)(c, 1, st));
      k_pty_pos_window<<<grid1(n), 256, 0, st>>>(t->O, t->p.obj_rows, t->p.obj_cols, t->win, t->order, t->iter, ns, k,
                                                  t->gw, rows, cols);
      PTY_RET(fft2(t, t->gw, t->dxy, false));
      const float nrm = (float)(1. / ((double)rows * cols));
      k_pty_pos_deriv<<<grid1(n), 256, 0, st>>>(t->dxy, rows, cols, std::sqrt(nrm), nrm);
      PTY_RET(fft2(t, t->dxy, t->dtmp, true, 2));
      k_pty_pos_probe<<<grid1(n), 256, 0, st>>>(t->dtmp, t->P, n);
      PTY_RET(fft2(t, t->dtmp, t->dxy, false, 2));
      k_pty_pos_partial<<<kRedBlocks, 256, 0, st>>>(t->fn, t->dxy, t->pats, t->pat_stride, t->p.use_bs ? t->bs : nullptr,
                                                    rows, cols, t->tl, a.norm, t->order, t->iter, ns, k, t->part,
                                                    t->cnt + 4, t->grad);
      PTY_CK(cudaGetLastError());
    }
    a.tw = t->tw_r;
    PTY_CK(t->kr.col(a, st));
    a.tw = t->tw_c;
    PTY_CK(t->kc.upd(a, st));
  }
  if (probe_phase) k_pty_add_step<<<grid1(n), 256, 0, st>>>(t->P, t->step, n);
  if (posupd) {   // util/ptycho.cpp:567-585: new shifts, mean removed, the object shifted by it
    k_pty_pos_update<<<1, 32, 0, st>>>(t->shifts, t->grad, t->scanpos, t->win, ns, (float)t->p.position_uncertainty,
                                       t->pmean);
    float2* objs[2] = {t->O, t->Op};
    for (float2* o : objs) {
      PTY_RET(fft2g(st, o, t->otmp, false, t->p.obj_rows, t->p.obj_cols, t->tw_or, t->tw_oc, t->orow, t->ocol, 1));
      k_pty_pos_oshift<<<grid1(on), 256, 0, st>>>(t->otmp, t->p.obj_rows, t->p.obj_cols, t->pmean);
      PTY_RET(fft2g(st, t->otmp, o, true, t->p.obj_rows, t->p.obj_cols, t->tw_or, t->tw_oc, t->orow, t->ocol, 1));
    }
    PTY_CK(cudaGetLastError());
  }
  if (probe_phase) {
    PTY_RET(angular_spectrum(t, t->P, true));
    if (zernike)   // util/ptycho.cpp:619-621: zernike_compute + zernike_reconstruct on the crop
      PTY_CK(zk_fit(t->P, t->p.rows, t->p.cols, (int)t->p.pupil_size, t->zk_tab, t->zk_part, t->zk_coef, st));
    else
      k_pty_pupil_mask<<<grid1(n), 256, 0, st>>>(t->P, t->p.rows, t->p.cols, (int)t->p.pupil_size);
    PTY_RET(angular_spectrum(t, t->P, false));
    PTY_RET(fft2(t, t->P, t->tmp, false));
    k_pty_far_part<<<kRedBlocks, 256, 0, st>>>(t->tmp, t->p.rows, t->p.cols, t->part, t->scal, t->cnt + 2);
    k_pty_mshift<<<grid1(n), 256, 0, st>>>(t->P, t->p.rows, t->p.cols, t->scal);
  }
  if (fista) {   // util/ptycho.cpp:665-667: FISTA_step(objectWave, objectWave, 1e-2)
    const float lam = 1e-2f;
    k_pty_fista<<<grid1(on), 256, 0, st>>>(t->O, t->fista, t->p.obj_rows, t->p.obj_cols,
                                            (float)(0.125 / (double)lam), lam);
    PTY_CK(cudaMemcpyAsync(t->O, t->fista, sizeof(float2) * on, cudaMemcpyDeviceToDevice, st));
  }
  if (t->p.mpie) {
    k_pty_csum<<<kRedBlocks, 256, 0, st>>>(t->O, t->msum, on, t->part, t->scal, t->cnt + 3, 0);
    k_pty_momentum<<<grid1(on), 256, 0, st>>>(t->O, t->Op, on, t->scal, t->coef, t->iter);
    if (probe_momentum) k_pty_probe_momentum<<<grid1(n), 256, 0, st>>>(t->P, t->Pp, n, t->coefz, t->iter);
  }
  k_pty_next<<<1, 1, 0, st>>>(t->iter);
  PTY_CK(cudaGetLastError());
  return CDX_OK;
}

// sweep kind of iteration `it`: phase 0 object, 1 probe, 2 probe with applyMod; + 3 with the
// FISTA object step (it < zernikeIter); + 6 with the probe momentum (dozernike with mPIE);
// + 12 with the Zernike pupil fit (dozernike in the probe phase); + 24 with the scan-position
// refinement (every 20 sweeps from 500 when position_uncertainty > 0)
bool pos_update(const cdx_pty* t, int it) {
  return t->p.position_uncertainty > 0 && it >= kPositionUpdateIter && it % 20 == 0;
}
int sweep_kind(const cdx_pty* t, int it) {
  const int phase = it < kUpdateProbeIter ? 0 : (it < kNoiseProjIter ? 1 : 2);
  const bool fista = it < t->p.zernike_iter;
  const bool dozernike = fista && it % 10 == 0;
  const bool pmom = dozernike && t->p.mpie;
  return phase + (fista ? 3 : 0) + (pmom ? 6 : 0) + (dozernike && phase > 0 ? 12 : 0) + (pos_update(t, it) ? 24 : 0);
}

int ensure_graph(cdx_pty* t, int kind) {
  cudaGraphExec_t& g = t->graph[kind];
  if (g) return CDX_OK;
  cudaGraph_t graph = nullptr;
  PTY_CK(cudaStreamBeginCapture(t->st, cudaStreamCaptureModeThreadLocal));
  const int phase = kind % 3;
  const int r = enqueue_sweep(t, phase >= 1, phase == 2, (kind / 3) % 2 == 1, (kind / 6) % 2 == 1, (kind / 12) % 2 == 1,
                              kind >= 24);
  const cudaError_t e = cudaStreamEndCapture(t->st, &graph);
  if (r != CDX_OK) {
    if (graph) cudaGraphDestroy(graph);
    return r;
  }
  PTY_CK(e);
  const cudaError_t ei = cudaGraphInstantiate(&g, graph, 0);
  cudaGraphDestroy(graph);
  PTY_CK(ei);
  return CDX_OK;
}

template <class T>
int dalloc(T** p, size_t count) {
  if (cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)) != cudaSuccess) {
    cudaGetLastError();
    return set_error(CDX_ERR_NOMEM, "device allocation failed (" + std::to_string(sizeof(T) * count) + " bytes)");
  }
  return CDX_OK;
}

}  // namespace

extern "C" {

int cdx_pty_params_default(cdx_pty_params* p) {
  if (!p) return set_error(CDX_ERR_ARG, "null params");
  std::memset(p, 0, sizeof *p);
  p->pupil_size = 500;
  p->beam_stop_size = 5;
  p->exposure = 1;
  p->mpie = 1;
  return CDX_OK;
}

int cdx_pty_scan_orders(int nscan, int n_iter, unsigned int seed, int* orders) {
  if (nscan < 1 || n_iter < 0 || !orders) return set_error(CDX_ERR_ARG, "bad scan-order arguments");
  scan_orders_host(nscan, n_iter, seed, orders);
  return CDX_OK;
}

int cdx_pty_create(const cdx_pty_params* p, void* stream, cdx_pty** out) {
  if (!p || !out) return set_error(CDX_ERR_ARG, "null argument");
  *out = nullptr;
  if (p->nscan < 1 || p->obj_rows < 1 || p->obj_cols < 1) return set_error(CDX_ERR_ARG, "bad scan count or object size");
  if (p->noise_level < 0 || !(p->position_uncertainty >= 0) || p->zernike_iter < 0)
    return set_error(CDX_ERR_ARG, "noise_level, position_uncertainty and zernike_iter must be >= 0");
  if (!(p->lambda > 0) || !(p->pixelsize > 0) || !(p->d > 0) || !(p->exposure > 0))
    return set_error(CDX_ERR_ARG, "lambda, d, pixelsize and exposure must be positive");
  const int pd = (int)p->pupil_size;
  if (pd < 1 || pd > p->rows || pd > p->cols)
    return set_error(CDX_ERR_ARG, "pupil_size must be in [1, min(rows, cols)] (the pupil crop reads inside the probe)");
  cdx_pty* t = new cdx_pty;
  t->p = *p;
  if (!pty_kernels(p->rows, t->kr) || !pty_kernels(p->cols, t->kc) || !row_launcher(p->cols) || !col_launcher(p->rows)) {
    delete t;
    return set_error(CDX_ERR_SIZE, "probe size must be 2^a 3^b in [16, 4096]");
  }
  auto fail = [&](int code) { cdx_pty_destroy(t); return code; };
  if (stream) t->st = (cudaStream_t)stream;
  else {
    if (cudaStreamCreateWithFlags(&t->st, cudaStreamNonBlocking) != cudaSuccess)
      return fail(set_error(CDX_ERR_CUDA, "stream creation failed"));
    t->own_st = true;
  }
  cudaError_t e = t->kr.prep();
  if (e == cudaSuccess) e = t->kc.prep();
  if (e == cudaSuccess) e = prep_launcher(p->rows)();
  if (e == cudaSuccess) e = prep_launcher(p->cols)();
  if (e != cudaSuccess) return fail(set_error(CDX_ERR_CUDA, std::string("kernel set-up: ") + cudaGetErrorString(e)));
  int r = device_twiddles(p->rows, &t->tw_r);
  if (r == CDX_OK) r = device_twiddles(p->cols, &t->tw_c);
  if (r != CDX_OK) return fail(r);
  t->tl = ilog2(t->kr.L);
  t->npx = (long long)p->rows * p->cols;
  t->onpx = (long long)p->obj_rows * p->obj_cols;
  const long long tiles = (p->cols + t->kr.L - 1) / t->kr.L;
  t->pat_stride = tiles * t->kr.L * p->rows;
  if ((r = dalloc(&t->O, t->onpx)) || (r = dalloc(&t->Op, t->onpx)) || (r = dalloc(&t->msum, t->onpx)) ||
      (r = dalloc(&t->P, t->npx)) || (r = dalloc(&t->step, t->npx)) || (r = dalloc(&t->tmp, t->npx)) ||
      (r = dalloc(&t->pupil, t->npx)) || (r = dalloc(&t->W, t->pat_stride)) ||
      (r = dalloc(&t->pats, t->pat_stride * p->nscan)) || (r = dalloc(&t->bs, t->pat_stride)) ||
      (r = dalloc(&t->win, p->nscan)) || (r = dalloc(&t->tpos, p->nscan)) || (r = dalloc(&t->iter, 1)) ||
      (r = dalloc(&t->scal, 1)) || (r = dalloc(&t->part, 3 * kRedBlocks)) || (r = dalloc(&t->cnt, 5)) || (r = dalloc(&t->derr, 1)) || (r = dalloc(&t->Pp, t->npx)) ||
      (r = dalloc(&t->fista, p->zernike_iter > 0 ? t->onpx : 1)))
    return fail(r);
  if (p->position_uncertainty > 0) {   // the refinement's buffers; the object transform if its size is supported
    const int ns2 = 2 * p->nscan;
    if ((r = dalloc(&t->shifts, ns2)) || (r = dalloc(&t->grad, ns2)) || (r = dalloc(&t->scanpos, ns2)) ||
        (r = dalloc(&t->pmean, 2)) || (r = dalloc(&t->fn, t->npx)) || (r = dalloc(&t->gw, t->npx)) ||
        (r = dalloc(&t->dxy, 2 * t->npx)) || (r = dalloc(&t->dtmp, 2 * t->npx)))
      return fail(r);
    t->orow = row_launcher(p->obj_cols);
    t->ocol = col_launcher(p->obj_rows);
    if (t->orow && t->ocol) {
      e = prep_launcher(p->obj_rows)();
      if (e == cudaSuccess) e = prep_launcher(p->obj_cols)();
      if (e != cudaSuccess) return fail(set_error(CDX_ERR_CUDA, std::string("object FFT set-up: ") + cudaGetErrorString(e)));
      if ((r = device_twiddles(p->obj_rows, &t->tw_or)) || (r = device_twiddles(p->obj_cols, &t->tw_oc)) ||
          (r = dalloc(&t->otmp, t->onpx)))
        return fail(r);
    }
  }
  if (p->zernike_iter > kUpdateProbeIter) {   // Zernike sweeps are possible: the fit's buffers and pixel table
    if ((r = dalloc(&t->zk_tab, (size_t)pd * pd)) || (r = dalloc(&t->zk_part, (size_t)zk_blocks(pd) * kZkModes)) ||
        (r = dalloc(&t->zk_coef, kZkModes)))
      return fail(r);
    if ((e = zk_table(t->zk_tab, pd, t->st)) != cudaSuccess)
      return fail(set_error(CDX_ERR_CUDA, std::string("Zernike table: ") + cudaGetErrorString(e)));
  }
  e = cudaMemsetAsync(t->W, 0, sizeof(float2) * t->pat_stride, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->pats, 0, sizeof(float) * t->pat_stride * p->nscan, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->bs, 0, sizeof(float) * t->pat_stride, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->step, 0, sizeof(float2) * t->npx, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->scal, 0, sizeof(PtyScal), t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->cnt, 0, sizeof(unsigned) * 5, t->st);
  if (e == cudaSuccess) e = cudaMemsetAsync(t->derr, 0, sizeof(int), t->st);
  if (e == cudaSuccess && p->use_bs) {
    k_pty_beamstop<<<grid1(t->npx), 256, 0, t->st>>>(t->bs, p->rows, p->cols, t->tl, (float)p->beam_stop_size);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventCreate(&t->e0);
  if (e == cudaSuccess) e = cudaEventCreate(&t->e1);
  if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
  if (e != cudaSuccess) return fail(set_error(CDX_ERR_CUDA, std::string("set-up: ") + cudaGetErrorString(e)));
  // propagate_pupil: lambda, distance dpupil, pixel size = resolution = lambda d / pixelsize / row
  // (util/ptycho.cpp:77-80, 231-233, 246), float members
  t->lam = (float)p->lambda;
  t->dist = (float)p->dpupil;
  t->res = (float)(p->lambda * p->d / p->pixelsize / p->rows);
  // propagate_esw: lambda, distance d, pixelsize, row (util/ptycho.cpp:74-76, 232)
  t->fresnel = p->is_fresnel ? cdx_fresnel_factor(p->lambda, p->d, p->pixelsize, p->rows, 0) : 0.f;
  *out = t;
  return CDX_OK;
}

int cdx_pty_destroy(cdx_pty* t) {
  if (!t) return CDX_OK;
  if (t->st) cudaStreamSynchronize(t->st);
  for (auto& g : t->graph)
    if (g) cudaGraphExecDestroy(g);
  void* bufs[] = {t->O, t->Op, t->P, t->step, t->W, t->tmp, t->pupil, t->pats, t->bs, t->msum, t->coef,
                  t->win, t->tpos, t->order, t->iter, t->scal, t->part, t->cnt, t->derr, t->Pp, t->fista,
                  t->coefz, t->zk_tab, t->zk_part, t->zk_coef, t->shifts, t->grad, t->scanpos, t->pmean, t->fn,
                  t->gw, t->dxy, t->dtmp, t->otmp};
  for (void* b : bufs)
    if (b) cudaFree(b);
  if (t->e0) cudaEventDestroy(t->e0);
  if (t->e1) cudaEventDestroy(t->e1);
  if (t->own_st && t->st) cudaStreamDestroy(t->st);
  delete t;
  return CDX_OK;
}

int cdx_pty_set_scan(cdx_pty* t, const float* posx, const float* posy) {
  if (!t || !posx || !posy) return set_error(CDX_ERR_ARG, "null argument");
  const int ns = t->p.nscan;
  std::vector<int2> w(ns), tp(ns);
  for (int i = 0; i < ns; ++i) {
    if (!std::isfinite(posx[i]) || !std::isfinite(posy[i]) || std::fabs(posx[i]) > 1e8f || std::fabs(posy[i]) > 1e8f)
      return set_error(CDX_ERR_ARG, "scan position not finite or out of range");
    w[i] = make_int2((int)std::round(posx[i]), (int)std::round(posy[i]));   // getWindow(round(posx), ...)
    tp[i] = make_int2((int)posx[i], (int)posy[i]);                          // addWindow(scanposx[i], ...)
  }
  PTY_CK(cudaMemcpyAsync(t->win, w.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice, t->st));
  PTY_CK(cudaMemcpyAsync(t->tpos, tp.data(), sizeof(int2) * ns, cudaMemcpyHostToDevice, t->st));
  t->win0 = w;
  if (t->scanpos) {   // scanposx then scanposy, for the refined window origins
    PTY_CK(cudaMemcpyAsync(t->scanpos, posx, sizeof(float) * ns, cudaMemcpyHostToDevice, t->st));
    PTY_CK(cudaMemcpyAsync(t->scanpos + ns, posy, sizeof(float) * ns, cudaMemcpyHostToDevice, t->st));
  }
  PTY_CK(cudaStreamSynchronize(t->st));
  t->have_scan = true;
  return CDX_OK;
}

int cdx_pty_set_patterns(cdx_pty* t, const float* patterns) {
  if (!t || !patterns) return set_error(CDX_ERR_ARG, "null argument");
  float* stage = nullptr;
  int r = dalloc(&stage, t->npx);
  if (r) return r;
  for (int i = 0; i < t->p.nscan && r == CDX_OK; ++i) {
    cudaError_t e = cudaMemcpyAsync(stage, patterns + (size_t)i * t->npx, sizeof(float) * t->npx,
                                    cudaMemcpyHostToDevice, t->st);
    if (e == cudaSuccess) {
      k_pty_tile<<<grid1(t->npx), 256, 0, t->st>>>(stage, t->pats + i * t->pat_stride, t->p.rows, t->p.cols, t->tl, 0);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
    if (e != cudaSuccess) r = set_error(CDX_ERR_CUDA, std::string("pattern upload: ") + cudaGetErrorString(e));
  }
  cudaFree(stage);
  if (r == CDX_OK) t->have_pats = true;
  return r;
}

int cdx_pty_get_patterns(cdx_pty* t, float* patterns) {
  if (!t || !patterns) return set_error(CDX_ERR_ARG, "null argument");
  float* stage = nullptr;
  int r = dalloc(&stage, t->npx);
  if (r) return r;
  for (int i = 0; i < t->p.nscan && r == CDX_OK; ++i) {
    k_pty_tile<<<grid1(t->npx), 256, 0, t->st>>>(t->pats + i * t->pat_stride, stage, t->p.rows, t->p.cols, t->tl, 1);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(patterns + (size_t)i * t->npx, stage, sizeof(float) * t->npx, cudaMemcpyDeviceToHost, t->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(t->st);
    if (e != cudaSuccess) r = set_error(CDX_ERR_CUDA, std::string("pattern download: ") + cudaGetErrorString(e));
  }
  cudaFree(stage);
  return r;
}

static int copy_c(cdx_pty* t, void* dst, const void* src, long long n, cudaMemcpyKind k) {
  PTY_CK(cudaMemcpyAsync(dst, src, sizeof(float2) * n, k, t->st));
  PTY_CK(cudaStreamSynchronize(t->st));
  return CDX_OK;
}

int cdx_pty_set_object(cdx_pty* t, const float* obj) {
  if (!t || !obj) return set_error(CDX_ERR_ARG, "null argument");
  PTY_RET(copy_c(t, t->O, obj, t->onpx, cudaMemcpyHostToDevice));
  t->have_obj = true;
  return CDX_OK;
}
int cdx_pty_get_object(cdx_pty* t, float* obj) {
  if (!t || !obj) return set_error(CDX_ERR_ARG, "null argument");
  return copy_c(t, obj, t->O, t->onpx, cudaMemcpyDeviceToHost);
}
int cdx_pty_set_probe(cdx_pty* t, const float* probe) {
  if (!t || !probe) return set_error(CDX_ERR_ARG, "null argument");
  PTY_RET(copy_c(t, t->P, probe, t->npx, cudaMemcpyHostToDevice));
  t->have_probe = true;
  return CDX_OK;
}
int cdx_pty_get_probe(cdx_pty* t, float* probe) {
  if (!t || !probe) return set_error(CDX_ERR_ARG, "null argument");
  return copy_c(t, probe, t->P, t->npx, cudaMemcpyDeviceToHost);
}
int cdx_pty_get_pupil(cdx_pty* t, float* pupil) {
  if (!t || !pupil) return set_error(CDX_ERR_ARG, "null argument");
  PTY_CK(cudaMemcpyAsync(t->pupil, t->P, sizeof(float2) * t->npx, cudaMemcpyDeviceToDevice, t->st));
  PTY_RET(angular_spectrum(t, t->pupil, true));
  return copy_c(t, pupil, t->pupil, t->npx, cudaMemcpyDeviceToHost);
}

int cdx_pty_set_pupil(cdx_pty* t, const float* pupil) {
  if (!t || !pupil) return set_error(CDX_ERR_ARG, "null argument");
  PTY_RET(copy_c(t, t->P, pupil, t->npx, cudaMemcpyHostToDevice));
  PTY_RET(angular_spectrum(t, t->P, false));
  PTY_CK(cudaStreamSynchronize(t->st));
  t->have_probe = true;
  return CDX_OK;
}

int cdx_pty_init_object(cdx_pty* t, unsigned long long seed) {
  if (!t) return set_error(CDX_ERR_ARG, "null argument");
  k_pty_random<<<grid1(t->onpx), 256, 0, t->st>>>(t->O, t->onpx, seed);
  k_pty_pupil_func<<<grid1(t->npx), 256, 0, t->st>>>(t->P, t->p.rows, t->p.cols, (float)t->p.pupil_size);
  PTY_CK(cudaGetLastError());
  PTY_RET(angular_spectrum(t, t->P, false));
  PTY_CK(cudaStreamSynchronize(t->st));
  t->have_obj = t->have_probe = true;
  return CDX_OK;
}

namespace {
int simulate(cdx_pty* t, bool ccd, unsigned long long seed) {
  if (!t->have_scan || !t->have_obj || !t->have_probe)
    return set_error(CDX_ERR_STATE, "scan positions, object and probe must be set first");
  const int ns = t->p.nscan;
  if (t->order_cap < ns) {
    if (t->order) cudaFree(t->order);
    t->order = nullptr;
    t->order_cap = 0;
    PTY_RET(dalloc(&t->order, ns));
    t->order_cap = ns;
  }
  std::vector<int> ident(ns);
  for (int i = 0; i < ns; ++i) ident[i] = i;
  PTY_CK(cudaMemcpyAsync(t->order, ident.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, t->st));
  PTY_CK(cudaMemsetAsync(t->iter, 0, sizeof(int), t->st));
  for (int k = 0; k < ns; ++k) {
    PtyArgs a = pass_args(t, k, false);
    a.tw = t->tw_c;
    PTY_CK(t->kc.fwd(a, t->st));
    ColArgs c{};
    c.in = t->W;
    c.out = t->tmp;
    c.in_tiled = 1;
    c.out_tiled = 0;
    c.in_stride = c.out_stride = t->npx;
    c.tw = t->tw_r;
    c.cols = t->p.cols;
    c.mode = COL_FFT;
    c.scale = 1.f;
    PTY_CK(col_launcher(t->p.rows)(c, 1, t->st));
    k_pty_sim_mod2<<<grid1(t->npx), 256, 0, t->st>>>(t->tmp, t->pats + k * t->pat_stride, t->p.rows, t->p.cols, t->tl,
                                                      (float)(1. / ((double)t->p.rows * t->p.cols)),
                                                      (float)t->p.exposure, (float)(1. / t->p.exposure),
                                                      t->p.use_bs ? t->bs : nullptr, ccd ? 1 : 0);
    PTY_CK(cudaGetLastError());
    if (ccd)   // ccdRecord(pattern, pattern, noiseLevel, devstates, exposure), then applyNorm(1/exposure)
      PTY_RET(cdx_ccd_record(t->pats + k * t->pat_stride, t->pat_stride, t->p.noise_level, (float)t->p.exposure,
                             (int)kRcolor, (float)(1. / t->p.exposure), seed ^ (0x9E3779B97F4A7C15ull * (k + 1)),
                             t->st));
  }
  PTY_CK(cudaStreamSynchronize(t->st));
  t->have_pats = true;
  return CDX_OK;
}
}  // namespace

int cdx_pty_simulate(cdx_pty* t) {
  if (!t) return set_error(CDX_ERR_ARG, "null argument");
  return simulate(t, false, 0);
}

int cdx_pty_simulate_ccd(cdx_pty* t, unsigned long long seed) {
  if (!t) return set_error(CDX_ERR_ARG, "null argument");
  return simulate(t, true, seed);
}

int cdx_pty_iterate(cdx_pty* t, int first_iter, int n_iter, const int* orders, unsigned int seed) {
  if (!t) return set_error(CDX_ERR_ARG, "null argument");
  if (first_iter < 0 || n_iter < 0) return set_error(CDX_ERR_ARG, "negative iteration index or count");
  if (first_iter + n_iter > kPositionUpdateIter && t->p.position_uncertainty > 0 && !(t->orow && t->ocol))
    return set_error(CDX_ERR_SIZE, "the scan-position refinement from iteration 500 (position_uncertainty > 0) "
                                   "shifts the object by FFT: object rows and cols must be 2^a 3^b in [16, 4096]");
  if (!t->have_scan || !t->have_pats || !t->have_obj || !t->have_probe)
    return set_error(CDX_ERR_STATE, "scan positions, patterns, object and probe must be set first");
  const int ns = t->p.nscan;
  std::vector<int> ord((size_t)std::max(1, n_iter) * ns);
  if (orders) {
    for (size_t i = 0; i < (size_t)n_iter * ns; ++i)
      if (orders[i] < 0 || orders[i] >= ns) return set_error(CDX_ERR_ARG, "scan order entry out of range");
    std::memcpy(ord.data(), orders, sizeof(int) * (size_t)n_iter * ns);
  } else {
    scan_orders_host(ns, n_iter, seed, ord.data());
  }
  // momentum coefficients (tk - 1)/tk+1 in the reference's float/double mix (util/ptycho.cpp:478, 677-680)
  std::vector<float> coef(std::max(1, n_iter)), coefz(std::max(1, n_iter));
  float tk = (float)(0.5 + std::sqrt(1.25));
  for (int i = 0; i < n_iter; ++i) {
    const float tkp1 = (float)(0.5 + std::sqrt(0.25 + (double)(tk * tk)));
    coef[i] = (tk - 1) / tkp1;
    coefz[i] = (float)((double)coef[i] * 0.8);   // (tk-1)/tkp1*0.8 (util/ptycho.cpp:684)
    tk = tkp1;
  }
  if (t->order_cap < (int)ord.size()) {
    if (t->order) cudaFree(t->order);
    t->order = nullptr;
    t->order_cap = 0;
    PTY_RET(dalloc(&t->order, ord.size()));
    t->order_cap = (int)ord.size();
    for (auto& g : t->graph)
      if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  }
  if (t->coef_cap < (int)coef.size()) {
    if (t->coef) cudaFree(t->coef);
    if (t->coefz) cudaFree(t->coefz);
    t->coef = t->coefz = nullptr;
    t->coef_cap = 0;
    PTY_RET(dalloc(&t->coef, coef.size()));
    PTY_RET(dalloc(&t->coefz, coef.size()));
    t->coef_cap = (int)coef.size();
    for (auto& g : t->graph)
      if (g) { cudaGraphExecDestroy(g); g = nullptr; }
  }
  cudaStream_t st = t->st;
  PTY_CK(cudaMemcpyAsync(t->order, ord.data(), sizeof(int) * ord.size(), cudaMemcpyHostToDevice, st));
  PTY_CK(cudaMemcpyAsync(t->coef, coef.data(), sizeof(float) * coef.size(), cudaMemcpyHostToDevice, st));
  PTY_CK(cudaMemcpyAsync(t->coefz, coefz.data(), sizeof(float) * coefz.size(), cudaMemcpyHostToDevice, st));
  // per-call state of iterate(): zero history and probe step, the overlap mask
  PTY_CK(cudaMemsetAsync(t->Op, 0, sizeof(float2) * t->onpx, st));
  PTY_CK(cudaMemsetAsync(t->step, 0, sizeof(float2) * t->npx, st));
  PTY_CK(cudaMemsetAsync(t->Pp, 0, sizeof(float2) * t->npx, st));
  if (t->shifts) {   // resetPosition (util/ptycho.cpp:299-303): zero shifts, the nominal windows
    PTY_CK(cudaMemsetAsync(t->shifts, 0, sizeof(float) * 2 * t->p.nscan, st));
    PTY_CK(cudaMemcpyAsync(t->win, t->win0.data(), sizeof(int2) * t->p.nscan, cudaMemcpyHostToDevice, st));
  }
  PTY_CK(cudaMemsetAsync(t->msum, 0, sizeof(float) * t->onpx, st));
  PTY_CK(cudaMemsetAsync(t->iter, 0, sizeof(int), st));
  k_pty_masksum<<<grid1(t->npx * ns), 256, 0, st>>>(t->msum, t->tpos, ns, t->p.rows, t->p.cols, t->p.obj_rows,
                                                     t->p.obj_cols, (float)(t->p.pupil_size / 2));
  k_pty_bitmap<<<grid1(t->onpx), 256, 0, st>>>(t->msum, t->onpx);
  PTY_CK(cudaGetLastError());
  for (int it = first_iter; it < first_iter + n_iter; ++it) PTY_RET(ensure_graph(t, sweep_kind(t, it)));
  PTY_CK(cudaEventRecord(t->e0, st));
  for (int it = first_iter; it < first_iter + n_iter; ++it)
    PTY_CK(cudaGraphLaunch(t->graph[sweep_kind(t, it)], st));
  // final global phase of the object (util/ptycho.cpp:731-735)
  k_pty_csum<<<kRedBlocks, 256, 0, st>>>(t->O, nullptr, t->onpx, t->part, t->scal, t->cnt + 3, 1);
  k_pty_conj_phase<<<grid1(t->onpx), 256, 0, st>>>(t->O, t->onpx, t->scal);
  PTY_CK(cudaGetLastError());
  PTY_CK(cudaEventRecord(t->e1, st));
  PTY_CK(cudaEventSynchronize(t->e1));
  PTY_CK(cudaEventElapsedTime(&t->last_ms, t->e0, t->e1));
  int h = 0;
  PTY_CK(cudaMemcpy(&h, t->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    PTY_CK(cudaMemset(t->derr, 0, sizeof(int)));
    return set_error(CDX_ERR_CUDA, "a column kernel's bulk staging copy timed out; the sweep results are invalid");
  }
  return CDX_OK;
}

int cdx_pty_last_ms(cdx_pty* t, float* ms) {
  if (!t || !ms) return set_error(CDX_ERR_ARG, "null argument");
  *ms = t->last_ms;
  return CDX_OK;
}

}  // extern "C"
