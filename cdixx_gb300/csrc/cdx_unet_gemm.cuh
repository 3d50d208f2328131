// Implicit-GEMM convolution kernels of the warm-start U-Net (sm_103a).
//
// Tensors are NHWC; convolution operands are BF16, accumulation FP32.  A
// convolution (kernel KH x KW, stride S, padding P) from X [N,H,W,Cin] to
// Y [N,Ho,Wo,Cout] with weights W [Cout][KH][KW][Cin] is three GEMMs:
//   forward   Y[m][co]   = sum_k  im2col(X)[m][k] W[co][k]        m = (n,oy,ox), k = (ky,kx,ci)
//   dgrad     dX[m'][ci] = sum_k' gather(dY)[m'][k'] Wt[ci][k']    m' = (n,iy,ix), k' = (ky,kx,co)
//   wgrad     dW[co][k]  = sum_m  dY[m][co] im2col(X)[m][k]
// with Wt [Cin][KH][KW][Cout] the transposed weights.  A transposed
// convolution is the adjoint: its forward is dgrad, its input gradient is
// forward and its weight gradient is wgrad with the roles of X and dY swapped.
// X may be the channel concatenation of two tensors (decoder skips): channels
// [0, C0) from x0, [C0, Cin) from x1; dgrad's output splits the same way.
//
// Tiles are staged in shared memory by 16-byte cp.async (8 channels, zero-
// filled outside the image or past K), fragments are read with ldmatrix
// (.trans for the transposed operands of wgrad), the products are
// mma.sync.m16n8k16 BF16 with FP32 accumulators.  Rows of a tile are 64 or
// 128 bytes with the 16-byte chunks XOR-swizzled so ldmatrix is conflict-free.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "cdx_umma.cuh"

namespace cdx {
namespace unet {

struct ConvShape {
  int N, H, W;        // input spatial size (of X)
  int Cin, C0;        // input channels (C0 from x0, Cin - C0 from x1)
  int Ho, Wo, Cout;   // output spatial size and channels
  int KH, KW, S, P;
};

struct GemmArgs {
  ConvShape s;
  const __nv_bfloat16* x0;   // forward/wgrad: X parts; dgrad: unused
  const __nv_bfloat16* x1;
  const __nv_bfloat16* dy;   // dgrad/wgrad: dY [N,Ho,Wo,Cout]
  const __nv_bfloat16* w;    // forward: W [Cout][K]; dgrad: Wt [Cin][K']
  float* out0;               // forward: Y; dgrad: dX part 0; wgrad: partials [split][Cout][K]
  float* out1;               // dgrad: dX part 1 (channels >= C0)
  int accumulate;            // forward/dgrad: add into the output
  int m_per_split;           // wgrad: output pixels per split
};

__device__ __forceinline__ void cp16(void* dst, const void* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit_g() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait_g() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(a));
}
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// byte offset of 16-byte chunk c of row r in a tile with 64-byte rows
__device__ __forceinline__ int sw64(int r, int c) { return r * 64 + ((c ^ ((r >> 1) & 3)) << 4); }
// ... with 128-byte rows
__device__ __forceinline__ int sw128(int r, int c) { return r * 128 + ((c ^ (r & 7)) << 4); }

// Source of the 8 channels starting at k of im2col(X) row (n, oy, ox); null outside.
__device__ __forceinline__ const __nv_bfloat16* im2col_src(const GemmArgs& a, int n, int oy, int ox, int k) {
  const ConvShape& s = a.s;
  const int kk = k / s.Cin, ci = k - kk * s.Cin;
  const int ky = kk / s.KW, kx = kk - ky * s.KW;
  if (ky >= s.KH) return nullptr;
  const int iy = oy * s.S - s.P + ky, ix = ox * s.S - s.P + kx;
  if (iy < 0 || iy >= s.H || ix < 0 || ix >= s.W) return nullptr;
  const long long pix = ((long long)n * s.H + iy) * s.W + ix;
  if (ci < s.C0) return a.x0 + pix * s.C0 + ci;
  const int c1 = s.Cin - s.C0;
  return a.x1 + pix * c1 + (ci - s.C0);
}
// Source of the 8 output channels starting at k' = (ky,kx,co) that reach input pixel (n, iy, ix).
__device__ __forceinline__ const __nv_bfloat16* dgrad_src(const GemmArgs& a, int n, int iy, int ix, int k) {
  const ConvShape& s = a.s;
  const int kk = k / s.Cout, co = k - kk * s.Cout;
  const int ky = kk / s.KW, kx = kk - ky * s.KW;
  if (ky >= s.KH) return nullptr;
  const int ty = iy + s.P - ky, tx = ix + s.P - kx;
  if (ty < 0 || tx < 0) return nullptr;
  const int oy = ty / s.S, ox = tx / s.S;
  if (oy * s.S != ty || ox * s.S != tx || oy >= s.Ho || ox >= s.Wo) return nullptr;
  return a.dy + (((long long)n * s.Ho + oy) * s.Wo + ox) * s.Cout + co;
}

// ------------------------------------------------------------ forward / dgrad
// CTA tile 128 x BN (BN = 64 or 32), K step 32, 4 warps (2 x 2), 3 stages.
template <bool DGRAD, int BN>
__global__ void __launch_bounds__(128) k_conv_gemm(GemmArgs a) {
  constexpr int BM = 128, BK = 32, ST = 3;
  constexpr int WN = BN / 2, NT = WN / 8;   // per-warp columns, n8 tiles
  __shared__ __align__(128) unsigned char sA[ST][BM * 64];
  __shared__ __align__(128) unsigned char sB[ST][BN * 64];
  const ConvShape& s = a.s;
  const int M = DGRAD ? s.N * s.H * s.W : s.N * s.Ho * s.Wo;
  const int NC = DGRAD ? s.Cin : s.Cout;                       // GEMM columns
  const int K = DGRAD ? s.KH * s.KW * s.Cout : s.KH * s.KW * s.Cin;
  const int KT = (K + BK - 1) / BK;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;

  // this thread stages row `tid` of the A tile: decode its pixel once
  const int am = m0 + tid;
  const bool arow = am < M;
  int an = 0, ay = 0, ax = 0;
  if (arow) {
    const int hw = DGRAD ? s.H * s.W : s.Ho * s.Wo, ww = DGRAD ? s.W : s.Wo;
    an = am / hw;
    const int r = am - an * hw;
    ay = r / ww;
    ax = r - ay * ww;
  }
  auto load = [&](int stage, int kt) {
    const int k0 = kt * BK;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int k = k0 + c * 8;
      const __nv_bfloat16* src = nullptr;
      if (arow && k < K) src = DGRAD ? dgrad_src(a, an, ay, ax, k) : im2col_src(a, an, ay, ax, k);
      cp16(sA[stage] + sw64(tid, c), src ? (const void*)src : (const void*)a.w, src != nullptr);
    }
#pragma unroll
    for (int i = 0; i < BN * 4 / 128; ++i) {
      const int q = tid + i * 128, r = q >> 2, c = q & 3;
      const int n = n0 + r, k = k0 + c * 8;
      const bool ok = n < NC && k < K;
      cp16(sB[stage] + sw64(r, c), ok ? (const void*)(a.w + (long long)n * K + k) : (const void*)a.w, ok);
    }
  };

  float acc[4][NT][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;

#pragma unroll
  for (int st = 0; st < ST - 1; ++st) {
    if (st < KT) load(st, st);
    cp_commit_g();
  }
  for (int kt = 0; kt < KT; ++kt) {
    cp_wait_g<ST - 2>();
    __syncthreads();
    if (kt + ST - 1 < KT) load((kt + ST - 1) % ST, kt + ST - 1);
    cp_commit_g();
    const unsigned char* tA = sA[kt % ST];
    const unsigned char* tB = sB[kt % ST];
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
      uint32_t af[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = wm * 64 + i * 16 + (lane & 15);
        ldsm_x4(af[i], tA + sw64(r, kk * 2 + (lane >> 4)));
      }
#pragma unroll
      for (int j = 0; j < NT; j += 2) {
        uint32_t bf[4];
        const int r = wn * WN + j * 8 + (lane & 7) + ((lane >> 4) << 3);
        ldsm_x4(bf, tB + sw64(r, kk * 2 + ((lane >> 3) & 1)));
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          mma16816(acc[i][j], af[i], bf[0], bf[1]);
          mma16816(acc[i][j + 1], af[i], bf[2], bf[3]);
        }
      }
    }
  }
  cp_wait_g<0>();
  // epilogue
  const int g = lane >> 2, q = lane & 3;
  const int c1 = s.Cin - s.C0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int m = m0 + wm * 64 + i * 16 + g + h * 8;
      if (m >= M) continue;
#pragma unroll
      for (int j = 0; j < NT; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int n = n0 + wn * WN + j * 8 + 2 * q + e;
          if (n >= NC) continue;
          const float v = acc[i][j][h * 2 + e];
          float* p;
          if (!DGRAD) p = a.out0 + (long long)m * s.Cout + n;
          else if (n < s.C0) p = a.out0 + (long long)m * s.C0 + n;
          else p = a.out1 + (long long)m * c1 + (n - s.C0);
          *p = a.accumulate ? *p + v : v;
        }
    }
}

// ------------------------------------------------------------------- wgrad
// CTA tile 64 (Cout) x 64 (K), reduction over a range of output pixels in
// steps of 32; partial sums per split, reduced in a fixed order afterwards.
__global__ void __launch_bounds__(128) k_conv_wgrad(GemmArgs a) {
  constexpr int BM = 64, BN = 64, BK = 32, ST = 3;
  __shared__ __align__(128) unsigned char sA[ST][BK * 128];   // dY rows (m) x 64 co
  __shared__ __align__(128) unsigned char sB[ST][BK * 128];   // im2col rows (m) x 64 k
  const ConvShape& s = a.s;
  const int M = s.N * s.Ho * s.Wo;
  const int K = s.KH * s.KW * s.Cin;
  const int co0 = blockIdx.y * BM, k0 = blockIdx.x * BN;
  const int mb = blockIdx.z * a.m_per_split;
  const int me = min(M, mb + a.m_per_split);
  const int KT = me > mb ? (me - mb + BK - 1) / BK : 0;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  const int hw = s.Ho * s.Wo;

  auto load = [&](int stage, int kt) {
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int q = tid + i * 128, r = q >> 3, c = q & 7;
      const int m = mb + kt * BK + r;
      // dY chunk: channels co0 + 8c .. +8 of pixel m
      const int co = co0 + c * 8;
      const bool oka = m < me && co < s.Cout;
      cp16(sA[stage] + sw128(r, c), oka ? (const void*)(a.dy + (long long)m * s.Cout + co) : (const void*)a.dy, oka);
      // im2col chunk: k0 + 8c .. +8 of pixel m
      const __nv_bfloat16* src = nullptr;
      const int k = k0 + c * 8;
      if (m < me && k < K) {
        const int n = m / hw, rr = m - n * hw, oy = rr / s.Wo, ox = rr - oy * s.Wo;
        src = im2col_src(a, n, oy, ox, k);
      }
      cp16(sB[stage] + sw128(r, c), src ? (const void*)src : (const void*)a.dy, src != nullptr);
    }
  };

  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][j][e] = 0.f;
#pragma unroll
  for (int st = 0; st < ST - 1; ++st) {
    if (st < KT) load(st, st);
    cp_commit_g();
  }
  for (int kt = 0; kt < KT; ++kt) {
    cp_wait_g<ST - 2>();
    __syncthreads();
    if (kt + ST - 1 < KT) load((kt + ST - 1) % ST, kt + ST - 1);
    cp_commit_g();
    const unsigned char* tA = sA[kt % ST];
    const unsigned char* tB = sB[kt % ST];
#pragma unroll
    for (int kk = 0; kk < 2; ++kk) {
      uint32_t af[2][4];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        // A'[co][m] = dY[m][co]^T: rows m = kk*16 + (lane&7) + 8*(lane>>4), chunk = co/8 + ((lane>>3)&1)
        const int r = kk * 16 + (lane & 7) + ((lane >> 4) << 3);
        const int c = (wm * 32 + i * 16) / 8 + ((lane >> 3) & 1);
        ldsm_x4_t(af[i], tA + sw128(r, c));
      }
#pragma unroll
      for (int j = 0; j < 4; j += 2) {
        uint32_t bf[4];
        // B'[m][k]: rows m = kk*16 + (lane&7) + 8*((lane>>3)&1), chunk = k/8 + (lane>>4)
        const int r = kk * 16 + (lane & 7) + (((lane >> 3) & 1) << 3);
        const int c = (wn * 32 + j * 8) / 8 + (lane >> 4);
        ldsm_x4_t(bf, tB + sw128(r, c));
#pragma unroll
        for (int i = 0; i < 2; ++i) {
          mma16816(acc[i][j], af[i], bf[0], bf[1]);
          mma16816(acc[i][j + 1], af[i], bf[2], bf[3]);
        }
      }
    }
  }
  cp_wait_g<0>();
  const int g = lane >> 2, q = lane & 3;
  float* part = a.out0 + (long long)blockIdx.z * s.Cout * K;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = co0 + wm * 32 + i * 16 + g + h * 8;
      if (co >= s.Cout) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int k = k0 + wn * 32 + j * 8 + 2 * q + e;
          if (k < K) part[(long long)co * K + k] = acc[i][j][h * 2 + e];
        }
    }
}

// ------------------------------------------------ tcgen05 operand policies
// The forward and data-gradient GEMMs on the 5th-generation tensor cores
// (cdx_umma.cuh): the same gathers as above, staged into the UMMA tiles.
struct ConvFwdOp {
  GemmArgs a;
  struct Row { int n, oy, ox; bool ok; };
  struct Kc { int ky, kx, ci; bool ok; };
  __device__ Row row(int m, int M) const {
    Row r{0, 0, 0, m < M};
    if (r.ok) {
      const int hw = a.s.Ho * a.s.Wo;
      r.n = m / hw;
      const int t = m - r.n * hw;
      r.oy = t / a.s.Wo;
      r.ox = t - r.oy * a.s.Wo;
    }
    return r;
  }
  __device__ Kc kc(int k, int K) const {
    const int kk = k / a.s.Cin, ci = k - kk * a.s.Cin, ky = kk / a.s.KW;
    return Kc{ky, kk - ky * a.s.KW, ci, k < K};
  }
  __device__ const __nv_bfloat16* a_src(const Row& r, const Kc& c) const {
    if (!r.ok || !c.ok) return nullptr;
    const ConvShape& s = a.s;
    const int iy = r.oy * s.S - s.P + c.ky, ix = r.ox * s.S - s.P + c.kx;
    if (iy < 0 || iy >= s.H || ix < 0 || ix >= s.W) return nullptr;
    const long long pix = ((long long)r.n * s.H + iy) * s.W + ix;
    if (c.ci < s.C0) return a.x0 + pix * s.C0 + c.ci;
    return a.x1 + pix * (s.Cin - s.C0) + (c.ci - s.C0);
  }
  __device__ const __nv_bfloat16* b_src(int n, int k) const {
    return a.w + (long long)n * (a.s.KH * a.s.KW * a.s.Cin) + k;
  }
  __device__ const void* dummy() const { return a.w; }
  __device__ void store(int m, int n0, const float* v, int cnt) const {
    float* p = a.out0 + (long long)m * a.s.Cout + n0;
    for (int j = 0; j < cnt; ++j) p[j] = a.accumulate ? p[j] + v[j] : v[j];
  }
};

struct ConvDgradOp {
  GemmArgs a;
  struct Row { int n, iy, ix; bool ok; };
  struct Kc { int ky, kx, co; bool ok; };
  __device__ Row row(int m, int M) const {
    Row r{0, 0, 0, m < M};
    if (r.ok) {
      const int hw = a.s.H * a.s.W;
      r.n = m / hw;
      const int t = m - r.n * hw;
      r.iy = t / a.s.W;
      r.ix = t - r.iy * a.s.W;
    }
    return r;
  }
  __device__ Kc kc(int k, int K) const {
    const int kk = k / a.s.Cout, co = k - kk * a.s.Cout, ky = kk / a.s.KW;
    return Kc{ky, kk - ky * a.s.KW, co, k < K};
  }
  __device__ const __nv_bfloat16* a_src(const Row& r, const Kc& c) const {
    if (!r.ok || !c.ok) return nullptr;
    const ConvShape& s = a.s;
    const int ty = r.iy + s.P - c.ky, tx = r.ix + s.P - c.kx;
    if (ty < 0 || tx < 0) return nullptr;
    const int oy = ty / s.S, ox = tx / s.S;
    if (oy * s.S != ty || ox * s.S != tx || oy >= s.Ho || ox >= s.Wo) return nullptr;
    return a.dy + (((long long)r.n * s.Ho + oy) * s.Wo + ox) * s.Cout + c.co;
  }
  __device__ const __nv_bfloat16* b_src(int n, int k) const {
    return a.w + (long long)n * (a.s.KH * a.s.KW * a.s.Cout) + k;
  }
  __device__ const void* dummy() const { return a.w; }
  __device__ void store(int m, int n0, const float* v, int cnt) const {
    const ConvShape& s = a.s;
    const int c1 = s.Cin - s.C0;
    for (int j = 0; j < cnt; ++j) {
      const int n = n0 + j;
      float* p = n < s.C0 ? a.out0 + (long long)m * s.C0 + n : a.out1 + (long long)m * c1 + (n - s.C0);
      *p = a.accumulate ? *p + v[j] : v[j];
    }
  }
};

}  // namespace unet
}  // namespace cdx
