// The Zernike pupil fit of the ptychographic probe phase (util/ptycho.cpp:617-626,
// src/gpu/beamDecomposition.cu:11-608): on a Zernike sweep the pd x pd crop of the
// back-propagated probe is projected on the real Zernike basis up to radial order
// 40 (861 modes), the coefficients are soft-thresholded and the crop is replaced
// by their sum, instead of being cut with the pupil disk.
//
// Device layout: a per-pixel table of the crop (covered fraction of the pixel in
// the disk of radius pd/2, the radius and angle of the covered part's centroid)
// built once per context, and the recurrence coefficients of the 441 radial
// polynomials in constant memory; per sweep three launches:
//   k_zk_project   four pixels per thread, the azimuthal orders split over four CTA
//                  rows; per mode a warp reduction, the CTA's four warps summed into
//                  one partial per (mode, pixel block)
//   k_zk_finish    one warp per mode sums its CTAs' partials in double, scales
//                  by 1/(pi (pd/2)^2) and soft-thresholds
//   k_zk_rebuild   the probe rewritten: the coefficients' sum inside the crop on
//                  the pixels the disk touches, zero elsewhere (crop, pad)
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "cdx_pty_zernike.cuh"

namespace cdx {
namespace {

constexpr int kZkThreads = 128;
constexpr int kZkWarps = kZkThreads / 32;
constexpr int kZkPix = 4;                                      // pixels per projection thread
constexpr int kZkRadial = (kZkMaxN / 2 + 1) * (kZkMaxN / 2 + 2) - (kZkMaxN / 2 + 1);   // 441 (m, n) pairs

// radial step (m, n) in mode order: R_n^m = (a rho^2 + b) R_{n-2}^m + c R_{n-4}^m, basis
// value R_n^m * nrm (nrm = sqrt(n+1) for m = 0, sqrt(2 (n+1)) otherwise)
struct ZkStep {
  float a, b, c, nrm;
};
__constant__ ZkStep c_zk[kZkRadial];

struct Cover {
  float a, cx, cy;
};

// compute_pixel (beamDecomposition.cu:11-104): area of the unit pixel centred at
// (px, py) inside the circle of radius r about the origin, and the centroid of
// that area.  Far pixels count 0 or 1; a pixel with all corners in (out) counts
// 1 (0); otherwise the polygon of the inside corners and the edge crossings,
// ordered by angle about the pixel centre, plus the circular segment beyond the
// chord when the circle crosses the pixel twice.
__device__ Cover pixel_cover(float px, float py, float r) {
  const float r2 = r * r;
  const float d2 = px * px + py * py;
  const float s2 = sqrtf(2.f);
  if (d2 > (r + s2) * (r + s2)) return {0.f, px, py};
  if (d2 < (r - s2) * (r - s2)) return {1.f, px, py};
  const float x0 = px - 0.5f, x1 = px + 0.5f, y0 = py - 0.5f, y1 = py + 0.5f;
  const float qx[4] = {x0, x1, x1, x0}, qy[4] = {y0, y0, y1, y1};
  bool in[4];
  int n_in = 0;
  for (int k = 0; k < 4; ++k) {
    in[k] = qx[k] * qx[k] + qy[k] * qy[k] < r2;
    n_in += in[k];
  }
  if (n_in == 4) return {1.f, px, py};
  if (n_in == 0) return {0.f, px, py};
  const float eps = 1e-5f;
  float ix[8], iy[8];
  int ni = 0;
  auto known = [&](float x, float y) {
    for (int k = 0; k < ni; ++k)
      if (fabsf(ix[k] - x) < eps && fabsf(iy[k] - y) < eps) return true;
    return false;
  };
  for (int e = 0; e < 2; ++e) {   // vertical edges x = x0, x1
    const float x = e ? x1 : x0;
    float val = (r - x) * (r + x);
    if (val >= -eps) {
      const float y = sqrtf(fmaxf(val, 0.f));
      if (y >= y0 - eps && y <= y1 + eps && !known(x, y)) { ix[ni] = x; iy[ni] = y; ++ni; }
      if (ni < 8 && y > eps && -y >= y0 - eps && -y <= y1 + eps && !known(x, -y)) { ix[ni] = x; iy[ni] = -y; ++ni; }
    }
  }
  for (int e = 0; e < 2; ++e) {   // horizontal edges y = y0, y1
    const float y = e ? y1 : y0;
    float val = (r - y) * (r + y);
    if (val >= -eps) {
      const float x = sqrtf(fmaxf(val, 0.f));
      if (x >= x0 - eps && x <= x1 + eps && !known(x, y)) { ix[ni] = x; iy[ni] = y; ++ni; }
      if (ni < 8 && x > eps && -x >= x0 - eps && -x <= x1 + eps && !known(-x, y)) { ix[ni] = -x; iy[ni] = y; ++ni; }
    }
  }
  float vx[12], vy[12], ang[12];
  int nv = 0;
  for (int k = 0; k < 4; ++k)
    if (in[k]) { vx[nv] = qx[k]; vy[nv] = qy[k]; ++nv; }
  for (int k = 0; k < ni; ++k) { vx[nv] = ix[k]; vy[nv] = iy[k]; ++nv; }
  if (nv < 3) return {n_in > 0 ? 1.f : 0.f, px, py};
  int idx[12];
  for (int k = 0; k < nv; ++k) {
    idx[k] = k;
    ang[k] = atan2f(vy[k] - py, vx[k] - px);
  }
  for (int i = 0; i < nv - 1; ++i)   // the reference's exchange sort by angle
    for (int j = i + 1; j < nv; ++j)
      if (ang[idx[i]] > ang[idx[j]]) { const int s = idx[i]; idx[i] = idx[j]; idx[j] = s; }
  float A = 0.f, Mx = 0.f, My = 0.f;
  for (int i = 0; i < nv; ++i) {
    const int a = idx[i], b = idx[(i + 1) % nv];
    const double cross = (double)vx[a] * vy[b] - (double)vx[b] * vy[a];
    A = (float)(A + cross);
    Mx = (float)(Mx + (vx[a] + vx[b]) * cross);
    My = (float)(My + (vy[a] + vy[b]) * cross);
  }
  A *= 0.5f;
  Mx /= 6.f;
  My /= 6.f;
  if (A < 0.f) { A = -A; Mx = -Mx; My = -My; }
  if (ni == 2) {   // circular segment between the chord and the arc
    const float mx = (ix[0] + ix[1]) * 0.5f, my = (iy[0] + iy[1]) * 0.5f;
    const float cx = ix[0] - ix[1], cy = iy[0] - iy[1];
    const float L = sqrtf(cx * cx + cy * cy);
    const float h = sqrtf(mx * mx + my * my);
    const float th = 2.f * atan2f(0.5f * L, h);
    float tms, shc;
    if (th < 1e-4f) {   // theta - sin(theta) and sin^3(theta/2) by their series
      const float t2 = th * th, t3 = t2 * th, t5 = t3 * t2;
      tms = t3 / 6.f - t5 / 120.f;
      const float sh = 0.5f * th;
      shc = sh * sh * sh;
    } else {
      tms = th - sinf(th);
      shc = powf(sinf(0.5f * th), 3.f);
    }
    const float As = 0.5f * r2 * tms;
    const float ds = tms > 1e-10f ? (4.f * r * shc) / (3.f * tms) : r;
    const float nrm = h > 1e-9f ? h : 1.f;
    A += As;
    Mx += As * ds * (mx / nrm);
    My += As * ds * (my / nrm);
  }
  if (A > 1e-9f) return {A, Mx / A, My / A};
  return {A, px, py};
}

// the crop's pixel table: x = column, y = row about ((pd-1)/2, (pd-1)/2), radius pd/2
__global__ void k_zk_table(float4* __restrict__ tab, int pd) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= pd * pd) return;
  const float c = (float)(pd - 1) / 2, rad = (float)pd / 2;
  const Cover cv = pixel_cover((float)(g % pd) - c, (float)(g / pd) - c, rad);
  float rho = 1.f, th = 0.f;
  if (cv.a > 2e-20f) {
    rho = fminf(sqrtf(cv.cx * cv.cx + cv.cy * cv.cy) / rad, 1.f);
    th = atan2f(cv.cy, cv.cx);
  }
  // x: projection weight (zero for pixels the disk misses), w: rebuilt (1) or zeroed (0)
  tab[g] = make_float4(cv.a > 2e-20f ? cv.a : 0.f, rho, th, cv.a < 2e-20f ? 0.f : 1.f);
}

// Visits the 861 modes in the reference's order (m = 0 .. 40; n = m, m+2 .. 40;
// cos then sin for m > 0) for P pixels at once: the radial polynomial times the
// pixel's weight from weight * rho^m by the three-term recurrence in n, times the
// normalisation; f(mode, z[P]) receives the basis values.
// Modes [mode0, mode1) are the azimuthal orders [m0, m1), whose radial steps start at j0.
template <int P, class F>
__device__ __forceinline__ void zk_walk(const float (&rho)[P], const float (&th)[P], const float (&wt)[P], F&& f,
                                        int m0 = 0, int m1 = kZkMaxN + 1, int mode0 = 0, int j0 = 0) {
  float rp[P], rr[P];
#pragma unroll
  for (int p = 0; p < P; ++p) {
    rp[p] = wt[p];
    rr[p] = rho[p] * rho[p];
    for (int m = 0; m < m0; ++m) rp[p] *= rho[p];
  }
  int mode = mode0, j = j0;
  for (int m = m0; m < m1; ++m) {
    float cm[P], sm[P], r2[P], r4[P];
#pragma unroll
    for (int p = 0; p < P; ++p) {
      cm[p] = 1.f;
      sm[p] = 0.f;
      if (m > 0) sincosf(m * th[p], &sm[p], &cm[p]);
      r2[p] = r4[p] = 0.f;
    }
    for (int n = m; n <= kZkMaxN; n += 2, ++j) {
      const ZkStep s = c_zk[j];
      float zc[P], zs[P];
#pragma unroll
      for (int p = 0; p < P; ++p) {
        const float cur = n == m ? rp[p] : fmaf(fmaf(s.a, rr[p], s.b), r2[p], s.c * r4[p]);
        r4[p] = r2[p];
        r2[p] = cur;
        const float z = cur * s.nrm;
        zc[p] = z * cm[p];
        zs[p] = z * sm[p];
      }
      f(mode++, zc);
      if (m > 0) f(mode++, zs);
    }
#pragma unroll
    for (int p = 0; p < P; ++p) rp[p] *= rho[p];
  }
}

// The projection's CTAs split the azimuthal orders into kZkGroups ranges of about equal mode
// counts (blockIdx.y), so a small crop still fills the GPU.
constexpr int kZkGroups = 4;
__device__ __forceinline__ void zk_group_range(int g, int& m0, int& m1, int& mode0, int& mode1, int& j0) {
  int m = 0, mode = 0, j = 0;
  auto advance_to = [&](int target) {
    while (m <= kZkMaxN && mode < target) {
      const int radial = (kZkMaxN - m) / 2 + 1;
      mode += radial * (m == 0 ? 1 : 2);
      j += radial;
      ++m;
    }
  };
  advance_to(g * kZkModes / kZkGroups);
  m0 = m;
  mode0 = mode;
  j0 = j;
  advance_to((g + 1) * kZkModes / kZkGroups);
  m1 = m;
  mode1 = mode;
}

__global__ void __launch_bounds__(kZkThreads) k_zk_project(const float2* __restrict__ P, int cols, int r0, int c0,
                                                            int pd, const float4* __restrict__ tab,
                                                            float2* __restrict__ part) {
  __shared__ float2 acc[kZkWarps][kZkModes];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int m0, m1, mode0, mode1, j0;
  zk_group_range(blockIdx.y, m0, m1, mode0, mode1, j0);
  float rho[kZkPix], th[kZkPix], wt[kZkPix];
  float2 v[kZkPix];
#pragma unroll
  for (int p = 0; p < kZkPix; ++p) {
    const int g = (blockIdx.x * kZkPix + p) * kZkThreads + threadIdx.x;
    float4 e = make_float4(0.f, 1.f, 0.f, 0.f);
    v[p] = make_float2(0.f, 0.f);
    if (g < pd * pd) {
      e = tab[g];
      if (e.x > 0.f) v[p] = P[(long long)(r0 + g / pd) * cols + c0 + g % pd];
    }
    wt[p] = e.x;
    rho[p] = e.y;
    th[p] = e.z;
  }
  zk_walk<kZkPix>(rho, th, wt, [&](int k, const float (&z)[kZkPix]) {
    float re = 0.f, im = 0.f;
#pragma unroll
    for (int p = 0; p < kZkPix; ++p) {
      re = fmaf(v[p].x, z[p], re);
      im = fmaf(v[p].y, z[p], im);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_xor_sync(0xffffffffu, re, o);
      im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    if (lane == 0) acc[warp][k] = make_float2(re, im);
  }, m0, m1, mode0, j0);
  __syncthreads();
  for (int k = mode0 + threadIdx.x; k < mode1; k += kZkThreads) {
    float2 s = acc[0][k];
#pragma unroll
    for (int w = 1; w < kZkWarps; ++w) {
      s.x += acc[w][k].x;
      s.y += acc[w][k].y;
    }
    part[(long long)k * gridDim.x + blockIdx.x] = s;
  }
}

// reduce_coefficients (norm 1/(pi r^2)) and regularize_zernike_coefficients as
// zernike_compute launches them (beamDecomposition.cu:460-513, 568-591): the
// launch passes the mode count (861) as the order bound, so mode k <= 430 is
// thresholded as (p, m) = (2k, 0) and mode k > 430 as (1 + 2 ((k - 431) / 2), 1);
// c *= max(0, 1 - (5e-5 p^2 + 5e-8 m^2) / |c|), zero for |c| <= 1e-9.
__global__ void k_zk_finish(const float2* __restrict__ part, int nblk, double norm, float2* __restrict__ coef) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= kZkModes) return;
  double sx = 0, sy = 0;
  for (int b = lane; b < nblk; b += 32) {
    const float2 p = part[(long long)k * nblk + b];
    sx += p.x;
    sy += p.y;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  if (lane) return;
  const float cx = (float)(sx * norm), cy = (float)(sy * norm);
  const int half = kZkModes >> 1;
  int p, m;
  if (k <= half) {
    p = 2 * k;
    m = 0;
  } else {
    m = 1;
    p = 1 + (((k - half - 1) >> 1) << 1);
  }
  const float factor = 5e-5f * p * p + 5e-8f * m * m;
  const float mag = hypotf(cx, cy);
  const float s = mag > 1e-9f ? fmaxf(0.f, 1.f - factor / mag) : 0.f;
  coef[k] = make_float2(cx * s, cy * s);
}

// zernike_reconstruct into the crop, then pad back: the whole probe is written
__global__ void k_zk_rebuild(float2* __restrict__ P, int rows, int cols, int r0, int c0, int pd,
                             const float4* __restrict__ tab, const float2* __restrict__ coef) {
  __shared__ float2 cs[kZkModes];
  for (int k = threadIdx.x; k < kZkModes; k += blockDim.x) cs[k] = coef[k];
  __syncthreads();
  const long long n = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / cols) - r0, y = (int)(i % cols) - c0;
    float2 out = make_float2(0.f, 0.f);
    if (x >= 0 && x < pd && y >= 0 && y < pd) {
      const float4 e = tab[x * pd + y];
      if (e.w > 0.f) {
        const float rho[1] = {e.y}, th[1] = {e.y > 2e-20f ? e.z : 0.f}, one[1] = {1.f};
        zk_walk<1>(rho, th, one, [&](int k, const float (&z)[1]) {
          out.x = fmaf(cs[k].x, z[0], out.x);
          out.y = fmaf(cs[k].y, z[0], out.y);
        });
      }
    }
    P[i] = out;
  }
}

}  // namespace

int zk_blocks(int pd) { return (pd * pd + kZkThreads * kZkPix - 1) / (kZkThreads * kZkPix); }

cudaError_t zk_table(float4* tab, int pd, cudaStream_t st) {
  // the recurrence of R_n^m in n (k1 R_n = (k2 rho^2 + k3) R_{n-2} + k4 R_{n-4}, the
  // coefficients of beamDecomposition.cu:162-176) divided through by k1, in double
  static const std::vector<ZkStep> steps = [] {
    std::vector<ZkStep> v;
    for (int m = 0; m <= kZkMaxN; ++m)
      for (int n = m; n <= kZkMaxN; n += 2) {
        ZkStep s{0.f, 0.f, 0.f, (float)std::sqrt(m == 0 ? n + 1.0 : 2.0 * (n + 1))};
        if (n == m + 2) {
          s.a = (float)(m + 2);
          s.b = (float)(-(m + 1));
        } else if (n > m + 2) {
          const double k1 = 0.5 * (n + m) * (n - m) * (n - 2.0), k2 = 2.0 * n * (n - 1.0) * (n - 2.0);
          const double k3 = -double(m) * m * (n - 1.0) - n * (n - 1.0) * (n - 2.0);
          const double k4 = -0.5 * n * (n + m - 2.0) * (n - m - 2.0);
          s.a = (float)(k2 / k1);
          s.b = (float)(k3 / k1);
          s.c = (float)(k4 / k1);
        }
        v.push_back(s);
      }
    return v;
  }();
  cudaError_t e = cudaMemcpyToSymbolAsync(c_zk, steps.data(), sizeof(ZkStep) * steps.size(), 0,
                                          cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  k_zk_table<<<(pd * pd + 127) / 128, 128, 0, st>>>(tab, pd);
  return cudaGetLastError();
}

cudaError_t zk_fit(float2* P, int rows, int cols, int pd, const float4* tab, float2* part, float2* coef,
                   cudaStream_t st) {
  const int r0 = (rows - pd) / 2, c0 = (cols - pd) / 2;
  const int nblk = zk_blocks(pd);
  k_zk_project<<<dim3(nblk, kZkGroups), kZkThreads, 0, st>>>(P, cols, r0, c0, pd, tab, part);
  const float rad = (float)pd / 2;
  k_zk_finish<<<(kZkModes + 7) / 8, 256, 0, st>>>(part, nblk, 1. / (M_PI * rad * rad), coef);
  const long long n = (long long)rows * cols;
  const int grid = (int)((n + 255) / 256 < 1216 ? (n + 255) / 256 : 1216);
  k_zk_rebuild<<<grid, 256, 0, st>>>(P, rows, cols, r0, c0, pd, tab, coef);
  return cudaGetLastError();
}

}  // namespace cdx
