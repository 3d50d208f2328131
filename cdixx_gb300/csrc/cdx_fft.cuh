// Shared-memory FFT engine for the CDI phase-retrieval kernels (sm_103a).
//
// A CTA holds L lines of length N in shared memory and transforms all of them
// with a self-sorting (Stockham, decimation-in-time) mixed-radix schedule:
// pass p with radix R and sub-length NS = R_0*...*R_{p-1} maps butterfly j
// (k = j mod NS) to
//     v_r = in[j + r*N/R] * W_{NS*R}^{r*k},   v = DFT_R(v),
//     out[(j-k)*R + k + r*NS] = v_r,
// which leaves the result in natural order.  Every pass is done in place:
// each thread first loads all of its butterflies into registers, the CTA
// synchronises, then the butterflies are computed and stored.
//
// The transform is the unnormalised DFT of cuFFT's C2C plans (forward
// exp(-2 pi i k n/N), inverse exp(+2 pi i k n/N)), which is what the reference
// calls through myFFT/myIFFT (src/gpu/cudaConfig.cu:175-180).  Twiddles come
// from a table W_N^t = exp(-2 pi i t/N) computed in double precision on the
// host and rounded once to float.
//
// Shared-memory layout: element i of line l sits at l*LD + i + (i >> 4), with
// LD = N + N/16 + 1.  The skew keeps the strided stores of the first pass and
// the column-tile loads free of bank conflicts for 64-bit accesses.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "cdx_umma.cuh"

namespace cdx {

#define CDX_HD __host__ __device__ __forceinline__

CDX_HD float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CDX_HD float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CDX_HD float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by -i (forward) or +i (inverse)
template <bool INV>
CDX_HD float2 rot90(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------- small DFTs
// The butterflies issue Blackwell's paired FP32 instructions (FADD2 / FFMA2,
// the __fadd2_rn / __ffma2_rn intrinsics of sm_100 and later): one instruction
// adds or fuses both components of a complex value, rounded exactly as two
// scalar operations would be, so the results are those of the scalar forms.
// Only lane-uniform operations pair up; a product with +-i swaps and negates one
// component, so those sums (add_rot / sub_rot) stay scalar.
CDX_HD float2 padd(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
CDX_HD float2 psub(float2 a, float2 b) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __fadd2_rn(a, make_float2(-b.x, -b.y));
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
// a * b + c per component, one rounding
CDX_HD float2 pfma(float2 a, float2 b, float2 c) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
  return __ffma2_rn(a, b, c);
#else
  return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}
// b + rot90(d) and b - rot90(d), rot90 the product with -i (forward) or +i (inverse)
template <bool INV>
CDX_HD float2 add_rot(float2 b, float2 d) {
  return INV ? make_float2(b.x - d.y, b.y + d.x) : make_float2(b.x + d.y, b.y - d.x);
}
template <bool INV>
CDX_HD float2 sub_rot(float2 b, float2 d) {
  return INV ? make_float2(b.x + d.y, b.y - d.x) : make_float2(b.x - d.y, b.y + d.x);
}

template <bool INV>
CDX_HD void dft2(float2& a, float2& b) {
  float2 t = a;
  a = padd(t, b);
  b = psub(t, b);
}

template <bool INV>
CDX_HD void dft3(float2* v) {
  const float s3 = 0.866025403784438647f;   // sqrt(3)/2
  float2 t1 = cadd(v[1], v[2]);
  float2 t2 = csub(v[1], v[2]);
  float2 m = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
  float2 r = rot90<INV>(make_float2(s3 * t2.x, s3 * t2.y));
  v[0] = cadd(v[0], t1);
  v[1] = cadd(m, r);
  v[2] = csub(m, r);
}

template <bool INV>
CDX_HD void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
  float2 a = padd(x0, x2), b = psub(x0, x2);
  float2 c = padd(x1, x3), d = psub(x1, x3);
  x0 = padd(a, c);
  x2 = psub(a, c);
  x1 = add_rot<INV>(b, d);
  x3 = sub_rot<INV>(b, d);
}

template <bool INV>
CDX_HD void dft8(float2* v) {
  const float h = 0.707106781186547524f;
  // even / odd radix-4 halves
  float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  float2 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  // W8^k o_k, k = 1..3 (forward: exp(-i pi k/4)): W8^1 o1 = h s1, W8^2 o2 = rot90(o2), W8^3 o3 = h s3
  const float2 s1 = INV ? make_float2(o1.x - o1.y, o1.x + o1.y) : make_float2(o1.x + o1.y, o1.y - o1.x);
  const float2 s3 = INV ? make_float2(-(o3.x + o3.y), o3.x - o3.y) : make_float2(o3.y - o3.x, -(o3.x + o3.y));
  const float2 hh = make_float2(h, h), mh = make_float2(-h, -h);
  v[0] = padd(e0, o0); v[4] = psub(e0, o0);
  v[1] = pfma(hh, s1, e1); v[5] = pfma(mh, s1, e1);
  v[2] = add_rot<INV>(e2, o2); v[6] = sub_rot<INV>(e2, o2);
  v[3] = pfma(hh, s3, e3); v[7] = pfma(mh, s3, e3);
}

template <bool INV>
CDX_HD void dft16(float2* v) {
  // 16 = 4 x 4: n = 4*n1 + n2, k = k1 + 4*k2
  const float c1 = 0.923879532511286756f;   // cos(pi/8)
  const float s1 = 0.382683432365089772f;   // sin(pi/8)
  const float h = 0.707106781186547524f;
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4<INV>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
  // after the inner DFTs, v[4*k1 + n2] holds A[n2][k1]; twiddle by W16^(n2*k1)
  const float sg = INV ? 1.f : -1.f;
  // (n2,k1) = (1,1): W16^1, (1,2): W16^2, (1,3): W16^3, (2,1): W16^2, (2,2): W16^4,
  // (2,3): W16^6, (3,1): W16^3, (3,2): W16^6, (3,3): W16^9
  const float2 w1 = make_float2(c1, sg * s1);
  const float2 w2 = make_float2(h, sg * h);
  const float2 w3 = make_float2(s1, sg * c1);
  const float2 w6 = make_float2(-h, sg * h);
  const float2 w9 = make_float2(-c1, -sg * s1);
  v[4 + 1] = cmul(v[4 + 1], w1);
  v[8 + 1] = cmul(v[8 + 1], w2);
  v[12 + 1] = cmul(v[12 + 1], w3);
  v[4 + 2] = cmul(v[4 + 2], w2);
  v[8 + 2] = rot90<INV>(v[8 + 2]);
  v[12 + 2] = cmul(v[12 + 2], w6);
  v[4 + 3] = cmul(v[4 + 3], w3);
  v[8 + 3] = cmul(v[8 + 3], w6);
  v[12 + 3] = cmul(v[12 + 3], w9);
  // outer DFTs over n2 for each k1; result X[k1 + 4*k2]
  float2 t[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    float2 a0 = v[4 * k1 + 0], a1 = v[4 * k1 + 1], a2 = v[4 * k1 + 2], a3 = v[4 * k1 + 3];
    dft4<INV>(a0, a1, a2, a3);
    t[k1 + 0] = a0; t[k1 + 4] = a1; t[k1 + 8] = a2; t[k1 + 12] = a3;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = t[i];
}

template <int R, bool INV>
CDX_HD void dftR(float2* v) {
  if constexpr (R == 2) dft2<INV>(v[0], v[1]);
  else if constexpr (R == 3) dft3<INV>(v);
  else if constexpr (R == 4) dft4<INV>(v[0], v[1], v[2], v[3]);
  else if constexpr (R == 8) dft8<INV>(v);
  else if constexpr (R == 16) dft16<INV>(v);
  else static_assert(R == 2, "unsupported radix");
}


// ---------------------------------------------------------------- plans
// The radices of length N, largest first: as many 16s as divide N, then 8, 4,
// 2, then 3s (radix(n, i) is the i-th; 0 past the last).
__host__ __device__ constexpr int radix_desc(int n, int i) {
  int m = n;
  int q = 0;
  while (m % 16 == 0) { if (q == i) return 16; m /= 16; ++q; }
  const int rs[3] = {8, 4, 2};
  for (int k = 0; k < 3; ++k)
    while (m % rs[k] == 0) { if (q == i) return rs[k]; m /= rs[k]; ++q; }
  while (m % 3 == 0) { if (q == i) return 3; m /= 3; ++q; }
  return 0;
}
__host__ __device__ constexpr int radix_count(int n) {
  int q = 0;
  while (radix_desc(n, q) != 0) ++q;
  return q;
}
// Radix of pass p for length N: the radices in a V, the 16s at both ends and
// the smaller radices in the middle.  The i-th radix of radix_desc (16s, then
// 8, 4, 2, then 3s) goes to the front for even i and to the back for odd i:
// 2048 = 16.8.16, 1024 = 16.4.16, 512 = 16.2.16, 384 = 16.3.8, 96 = 16.3.2,
// 3072 = 16.4.3.16.  Measured per 4.2 M-pixel iteration against
// the largest-first order (16.16.8 etc.): 2048^2 -4.7 %, 1024^2 x4 -12.5 %,
// 512^2 x16 -5.9 %, 384^2 x16 -3.5 %; a V that reads the same both ways is
// also the inverse order, so both transforms share one twiddle table.
__host__ __device__ constexpr int plan_radix(int n, int p) {
  const int m = radix_count(n);
  if (p < 0 || p >= m) return 0;
  const int front = (m + 1) / 2;   // positions 0..front-1 take the even ranks in order
  return p < front ? radix_desc(n, 2 * p) : radix_desc(n, 2 * (m - 1 - p) + 1);
}
__host__ __device__ constexpr int plan_ns(int n, int p) {
  int ns = 1;
  for (int i = 0; i < p; ++i) ns *= plan_radix(n, i);
  return ns;
}
__host__ __device__ constexpr bool size_supported(int n) {
  if (n < 16) return false;
  int m = n;
  while (m % 2 == 0) m /= 2;
  while (m % 3 == 0) m /= 3;
  return m == 1;
}
__host__ __device__ constexpr int plan_len(int n) {
  int q = 0;
  while (plan_radix(n, q) != 0) ++q;
  return q;
}
// Two schedules per length: plan 0 is the order above, plan 1 the same radices
// reversed.  A transform with plan 0 ends with the radix plan 1 starts with,
// and its last pass leaves a thread's values exactly where plan 1's first pass
// reads them, so two transforms chained through an element-wise step hand the
// data over in registers.
__host__ __device__ constexpr int plan_radix_x(int n, int plan, int p) {
  return plan == 0 ? plan_radix(n, p) : (p < plan_len(n) ? plan_radix(n, plan_len(n) - 1 - p) : 0);
}
__host__ __device__ constexpr int plan_ns_x(int n, int plan, int p) {
  int ns = 1;
  for (int i = 0; i < p; ++i) ns *= plan_radix_x(n, plan, i);
  return ns;
}
// Twiddles of pass p live in a block of (R-1)*NS entries, entry (r-1)*NS + k
// = W_N^(r*k*N/(NS*R)) for r = 1..R-1, k < NS, so the threads of a warp (k
// consecutive, r fixed) read consecutive words.  Pass 0 (NS = 1) needs none.
// The table of a length holds plan 0's blocks, then plan 1's; when the plans
// are the same sequence (a symmetric V) plan 1 reads plan 0's blocks.
__host__ __device__ constexpr bool plans_same(int n) {
  for (int p = 0; p < plan_len(n); ++p)
    if (plan_radix_x(n, 0, p) != plan_radix_x(n, 1, p)) return false;
  return true;
}
__host__ __device__ constexpr int tw_plan_count(int n, int plan) {
  int off = 0;
  for (int q = 1; q < plan_len(n); ++q) off += (plan_radix_x(n, plan, q) - 1) * plan_ns_x(n, plan, q);
  return off;
}
__host__ __device__ constexpr int tw_offset_x(int n, int plan, int p) {
  int off = (plan == 0 || plans_same(n)) ? 0 : tw_plan_count(n, 0);
  for (int q = 1; q < p; ++q) off += (plan_radix_x(n, plan, q) - 1) * plan_ns_x(n, plan, q);
  return off;
}
__host__ __device__ constexpr int tw_offset(int n, int p) { return tw_offset_x(n, 0, p); }
__host__ __device__ constexpr int tw_count(int n) {
  return tw_plan_count(n, 0) + (plans_same(n) ? 0 : tw_plan_count(n, 1));
}

__host__ __device__ constexpr int pow2_floor(int x) {
  int p = 1;
  while (p * 2 <= x) p *= 2;
  return p;
}

// Launch geometry per length: T threads, L lines per CTA (a power of two >= 2,
// so a tile of L columns has a power-of-two width and a row CTA moves at least
// 32-byte pieces of it), about 16 complex values per thread and pass (32 at
// N = 4096).  Small CTAs keep three or more resident per SM.
template <int N>
struct Geom {
  static constexpr int T = N >= 3072 ? 512 : 256;
  static constexpr int MINB = T == 512 ? 1 : 3;   // resident CTAs per SM the register budget targets
  static constexpr int ELEMS = 16 * T;
  static constexpr int L = pow2_floor((ELEMS / N) < 2 ? 2 : (ELEMS / N));
  static constexpr int LOG2L = L == 1 ? 0 : (L == 2 ? 1 : (L == 4 ? 2 : (L == 8 ? 3 : (L == 16 ? 4 : (L == 32 ? 5 :
                               (L == 64 ? 6 : (L == 128 ? 7 : 8)))))));
  // line stride in float2: >= N + N/16, and for L < 16 congruent to 16/L mod 16
  // so a tile row (L consecutive lines at one index) hits distinct bank pairs;
  // odd otherwise.
  static constexpr int BASE = N + (N >> 4);
  static constexpr int WANT = (L < 16) ? (16 / L) : 1;
  static constexpr int LD = BASE + (((WANT - BASE) % 16) + 16) % 16 + ((L < 16) ? 0 : (((BASE + ((((WANT - BASE) % 16) + 16) % 16)) % 2 == 0) ? 1 : 0));
  static constexpr int TWN = tw_count(N);
  // shared memory: the L lines; ROW_ITER adds L rows of rho (8 B/px), COL_ITER
  // sqrt(I) (4 B/px) and, for the noise-tolerant projection, I and the beamstop
  static constexpr int SMEM_LINES = L * LD * (int)sizeof(float2);
  static constexpr int SMEM_ROW_ITER = SMEM_LINES + L * N * (int)sizeof(float2) + L * ((N + 31) >> 5) * 4;
  static constexpr int SMEM_COL_ITER = SMEM_LINES + L * N * (int)sizeof(float);
  static constexpr int SMEM_COL_CCD = SMEM_LINES + 3 * L * N * (int)sizeof(float);
  static constexpr int SMEM_MAX = SMEM_ROW_ITER > SMEM_COL_CCD ? SMEM_ROW_ITER : SMEM_COL_CCD;
  __device__ __forceinline__ static int idx(int l, int i) { return l * LD + i + (i >> 4); }
};

// One Stockham pass over the L lines of Geom<N>.
template <int N, int P, bool INV>
__device__ __forceinline__ void fft_pass(float2* buf, const float2* tw) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  constexpr int R = plan_radix(N, P);
  constexpr int NS = plan_ns(N, P);
  constexpr int NR = N / R;
  constexpr int NB = L * NR;
  constexpr int B = (NB + T - 1) / T;
  float2 v[B][R];
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int g = threadIdx.x + b * T;
    if ((NB % T) == 0 || g < NB) {
      const int l = g / NR, j = g - l * NR;
#pragma unroll
      for (int r = 0; r < R; ++r) v[b][r] = buf[G::idx(l, j + r * NR)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < B; ++b) {
    const int g = threadIdx.x + b * T;
    if ((NB % T) == 0 || g < NB) {
      const int l = g / NR, j = g - l * NR;
      const int k = j % NS;
      if constexpr (NS > 1) {
        const float2* twp = tw + tw_offset(N, P);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(twp + (r - 1) * NS + k);
          if (INV) w.y = -w.y;
          v[b][r] = cmul(v[b][r], w);
        }
      }
      dftR<R, INV>(v[b]);
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) buf[G::idx(l, base + r * NS)] = v[b][r];
    }
  }
  __syncthreads();
}

// ------------------------------------------------------- tensor-core radix 16
// The DFT-16 of eight butterflies at once as warp MMAs (mma.sync m16n8k16,
// BF16 operands, FP32 accumulation).  In real form
//     [Yr; Yi] = [[Fr, -Fi], [Fi, Fr]] [Xr; Xi],   F[m][r] = exp(-+2 pi i m r/16),
// i.e. two 16-row tiles (Yr, Yi) times two 16-deep K steps (Xr, Xi), each an
// m16n8k16 MMA with the 8 butterflies as the N dimension.  Every operand is
// split into a BF16 head and a BF16 tail (x = hi + lo + O(2^-16 x)); the
// three products hi*hi + hi*lo + lo*hi are accumulated in FP32 (the lo*lo term,
// O(2^-16), is dropped), 12 MMAs per 8 butterflies.  Relative error of a pass
// ~1e-5: a lower-precision path, reported against the float64 oracle.
//
// Fragment layouts of mma.m16n8k16 (PTX ISA): with g = lane/4, q = lane%4,
//   A (16x16, row): {a0,a1} = A[g][2q..2q+1], {a2,a3} = A[g+8][2q..], {a4,a5} = A[g][2q+8..], {a6,a7} = A[g+8][2q+8..]
//   B (16x8, col):  {b0,b1} = B[2q..2q+1][g], {b2,b3} = B[2q+8..2q+9][g]
//   C (16x8):       {c0,c1} = C[g][2q..2q+1], {c2,c3} = C[g+8][2q..2q+1]
struct BF2 {
  uint32_t hi, lo;
};
__device__ __forceinline__ BF2 split_bf16x2(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  BF2 r;
  r.hi = *reinterpret_cast<uint32_t*>(&h);
  r.lo = *reinterpret_cast<uint32_t*>(&l);
  return r;
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// A fragments of Fr, Fi (head and tail) for this lane; sgn = -1 forward, +1 inverse.
struct DftFrag {
  uint32_t fr_hi[4], fr_lo[4], fi_hi[4], fi_lo[4], nfi_hi[4], nfi_lo[4];
};
template <bool INV>
__device__ __forceinline__ void dft16_fragments(DftFrag& f) {
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  const float sgn = INV ? 1.f : -1.f;
  // register i of the fragment holds rows (g, g+8) x cols (2q, 2q+1) / (2q+8, 2q+9)
  const int rows[4] = {g, g + 8, g, g + 8};
  const int cols[4] = {2 * q, 2 * q, 2 * q + 8, 2 * q + 8};
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    float cr[2], ci[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      float s, c;
      sincospif((float)((rows[i] * (cols[i] + e)) & 15) / 8.f, &s, &c);   // angle 2 pi m r / 16
      cr[e] = c;
      ci[e] = sgn * s;
    }
    BF2 r = split_bf16x2(cr[0], cr[1]);
    BF2 m = split_bf16x2(ci[0], ci[1]);
    BF2 n = split_bf16x2(-ci[0], -ci[1]);
    f.fr_hi[i] = r.hi; f.fr_lo[i] = r.lo;
    f.fi_hi[i] = m.hi; f.fi_lo[i] = m.lo;
    f.nfi_hi[i] = n.hi; f.nfi_lo[i] = n.lo;
  }
}

// D += A * X with A, X split into head and tail (three products).
__device__ __forceinline__ void mma3(float (&d)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4],
                                     uint32_t bh0, uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  mma_bf16(d, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  mma_bf16(d, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  mma_bf16(d, al[0], al[1], al[2], al[3], bh0, bh1);
}

// One radix-16 Stockham pass (same index map as fft_pass) with the DFTs on the
// tensor cores.  Butterflies are taken 8 at a time per warp.
template <int N, int P, bool INV>
__device__ __forceinline__ void fft_pass_tc16(float2* buf, const float2* tw, const DftFrag& F) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  constexpr int R = 16;
  static_assert(plan_radix(N, P) == 16, "tensor-core pass is radix 16");
  constexpr int NS = plan_ns(N, P);
  constexpr int NR = N / R;
  constexpr int NB = L * NR;
  static_assert(NB % 8 == 0, "butterflies come in groups of 8");
  constexpr int CHUNKS = NB / 8;
  constexpr int WARPS = T / 32;
  constexpr int CPW = (CHUNKS + WARPS - 1) / WARPS;   // chunks per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, q = lane & 3;
  // this lane loads components r = 2q, 2q+1, 2q+8, 2q+9 of butterfly g of each chunk
  float2 x[CPW][4];
#pragma unroll
  for (int c = 0; c < CPW; ++c) {
    const int ch = warp + c * WARPS;
    if (CHUNKS % WARPS == 0 || ch < CHUNKS) {
      const int bfly = ch * 8 + g;
      const int l = bfly / NR, j = bfly - l * NR;
      const int k = j % NS;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int r = 2 * q + (e & 1) + ((e >> 1) << 3);
        float2 v = buf[G::idx(l, j + r * NR)];
        if constexpr (NS > 1) {
          if (r > 0) {
            float2 w = __ldg(tw + tw_offset(N, P) + (r - 1) * NS + k);
            if (INV) w.y = -w.y;
            v = cmul(v, w);
          }
        }
        x[c][e] = v;
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int c = 0; c < CPW; ++c) {
    const int ch = warp + c * WARPS;
    if (CHUNKS % WARPS == 0 || ch < CHUNKS) {
      // B fragments: Xr rows (2q, 2q+1 | 2q+8, 2q+9) of column g, and Xi
      const BF2 xr01 = split_bf16x2(x[c][0].x, x[c][1].x), xr89 = split_bf16x2(x[c][2].x, x[c][3].x);
      const BF2 xi01 = split_bf16x2(x[c][0].y, x[c][1].y), xi89 = split_bf16x2(x[c][2].y, x[c][3].y);
      float yr[4] = {0.f, 0.f, 0.f, 0.f}, yi[4] = {0.f, 0.f, 0.f, 0.f};
      mma3(yr, F.fr_hi, F.fr_lo, xr01.hi, xr89.hi, xr01.lo, xr89.lo);     // Yr += Fr Xr
      mma3(yr, F.nfi_hi, F.nfi_lo, xi01.hi, xi89.hi, xi01.lo, xi89.lo);   // Yr -= Fi Xi
      mma3(yi, F.fi_hi, F.fi_lo, xr01.hi, xr89.hi, xr01.lo, xr89.lo);     // Yi += Fi Xr
      mma3(yi, F.fr_hi, F.fr_lo, xi01.hi, xi89.hi, xi01.lo, xi89.lo);     // Yi += Fr Xi
      // this lane holds Y[m][n] for m in {g, g+8}, butterflies n in {2q, 2q+1}
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int m = g + ((e >> 1) << 3), n = 2 * q + (e & 1);
        const int bfly = ch * 8 + n;
        const int l = bfly / NR, j = bfly - l * NR;
        const int k = j % NS;
        buf[G::idx(l, (j - k) * R + k + m * NS)] = make_float2(yr[e], yi[e]);
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------- tcgen05 (UMMA) radix 16
// The DFT-16 of every butterfly of a pass on the 5th-generation tensor cores.
// Thread t owns butterfly t (rows of 128-butterfly tiles, NT = T/128 tiles).
// Its 16 twiddled inputs are split into BF16 heads and tails and written as
// one 128-byte row of the tile's A operand, K-major SWIZZLE_128B:
//     A[t] = [Xr_hi(16) | Xi_hi(16) | Xr_lo(16) | Xi_lo(16)]        (K = 64)
// The DFT matrix in real form G (32 outputs x 32 inputs: Yr = Fr Xr - Fi Xi,
// Yi = Fi Xr + Fr Xi), split the same way, is the B operand twice:
//     Bm[n] = [G_hi(n, :) | G_hi(n, :)]   (K = 64),   Bl[n] = G_lo(n, :)  (K = 32)
// so D = A Bm^T + A[:, 0:32] Bl^T = X_hi G_hi + X_lo G_hi + X_hi G_lo, the
// compensated product (the tail x tail term, O(2^-16), dropped) in six
// m128n32k16 MMAs per tile, FP32 accumulation in TMEM (32 columns per tile).
// One elected thread issues them and commits to an mbarrier; warp w then
// reads its 32 butterflies' rows (TMEM lanes 32 (w % 4) .., columns of tile
// w / 4) with one tcgen05.ld.32x32b.x32: each thread gets Yr[0..15], Yi[0..15]
// of its own butterfly and stores them to the Stockham positions.
// Every wait is bounded (umma::kSpinLimit polls); a wait that runs out sets
// bit 0 of *err, and the kernel carries on to its end (results invalid).
struct UmmaFft {
  unsigned a;       // shared address of the NT A tiles (16 KB each, 1024-aligned)
  unsigned bm, bl;  // shared addresses of Bm and Bl (4 KB each, 1024-aligned) for the current direction
  unsigned tmem;    // TMEM base (32 columns per tile)
  unsigned bar;     // mbarrier (one arrival per pass)
  unsigned phase;   // parity of the next completion
  int* err;
};
constexpr int kUmmaTileBytes = 128 * 128;
constexpr int kUmmaBBytes = 32 * 128;

// G_hi / G_lo rows for direction INV into Bm and Bl (SW128 K-major): entry
// (n, k) of G is +-cos or +-sin of 2 pi q / 16, q = m r mod 16, from float
// values of cos(pi j/8) (float rounding of the exact constants), split.
template <bool INV, int T>
__device__ __forceinline__ void umma_dft16_b(const UmmaFft& U, unsigned char* smem_base) {
  const float c1 = 0.923879532511286756f, s1 = 0.382683432365089772f, h = 0.707106781186547524f;
  const float c16[16] = {1.f, c1, h, s1, 0.f, -s1, -h, -c1, -1.f, -c1, -h, -s1, 0.f, s1, h, c1};
  const float sg = INV ? 1.f : -1.f;
  unsigned char* bm = smem_base + (U.bm - (unsigned)__cvta_generic_to_shared(smem_base));
  unsigned char* bl = smem_base + (U.bl - (unsigned)__cvta_generic_to_shared(smem_base));
  // 32 rows x 8 chunks of 8 BF16: thread t fills (row, chunk) pairs t, t + T, ...
  for (int q = threadIdx.x; q < 32 * 8; q += T) {
    const int n = q >> 3, ch = q & 7;
    const int m = n & 15;
    __align__(16) __nv_bfloat16 hv[8], lv[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int k = ((ch & 3) << 3) + e;   // input index 0..31 (k < 16: Xr[k], else Xi[k - 16])
      const int r = k & 15, qq = (m * r) & 15;
      const float cs = c16[qq], sn = sg * c16[(qq + 12) & 15];   // Fr, Fi
      float g;
      if (n < 16) g = k < 16 ? cs : -sn;   // Yr row
      else g = k < 16 ? sn : cs;           // Yi row
      const __nv_bfloat16 hi = __float2bfloat16_rn(g);
      hv[e] = hi;
      lv[e] = __float2bfloat16_rn(g - __bfloat162float(hi));
    }
    // Bm: chunks 0-3 and 4-7 both hold G_hi; Bl: chunks 0-3 hold G_lo (4-7 unused)
    *reinterpret_cast<uint4*>(bm + umma::sw128(n, ch)) = *reinterpret_cast<const uint4*>(hv);
    if (ch < 4) *reinterpret_cast<uint4*>(bl + umma::sw128(n, ch)) = *reinterpret_cast<const uint4*>(lv);
  }
}

template <int N, int P, bool INV>
__device__ __forceinline__ void fft_pass_umma16(float2* buf, const float2* tw, UmmaFft& U, unsigned char* smem_base) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  constexpr int R = 16;
  static_assert(plan_radix(N, P) == 16, "tensor-core pass is radix 16");
  constexpr int NS = plan_ns(N, P);
  constexpr int NR = N / R;
  constexpr int NB = L * NR;
  static_assert(NB <= T && T % 128 == 0, "one butterfly per thread, whole 128-row tiles");
  constexpr int NT = T / 128;
  const int t = threadIdx.x, warp = t >> 5;
  const bool mine = NB == T || t < NB;
  int l = 0, j = 0, k = 0;
  float2 x[16];
  if (mine) {
    l = t / NR;
    j = t - l * NR;
    k = j % NS;
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      float2 v = buf[G::idx(l, j + r * NR)];
      if constexpr (NS > 1) {
        if (r > 0) {
          float2 w = __ldg(tw + tw_offset(N, P) + (r - 1) * NS + k);
          if (INV) w.y = -w.y;
          v = cmul(v, w);
        }
      }
      x[r] = v;
    }
  } else {
#pragma unroll
    for (int r = 0; r < 16; ++r) x[r] = make_float2(0.f, 0.f);
  }
  // A row: chunks 0-1 Xr_hi, 2-3 Xi_hi, 4-5 Xr_lo, 6-7 Xi_lo (8 BF16 each)
  {
    unsigned char* arow = smem_base + (U.a - (unsigned)__cvta_generic_to_shared(smem_base)) + (t >> 7) * kUmmaTileBytes;
    const int row = t & 127;
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      uint32_t rh[4], ih[4], rl[4], il[4];   // packed pairs (element 2e in the low half)
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float2 v0 = x[half * 8 + 2 * e], v1 = x[half * 8 + 2 * e + 1];
        const BF2 re = split_bf16x2(v0.x, v1.x), im = split_bf16x2(v0.y, v1.y);
        rh[e] = re.hi;
        rl[e] = re.lo;
        ih[e] = im.hi;
        il[e] = im.lo;
      }
      *reinterpret_cast<uint4*>(arow + umma::sw128(row, 0 + half)) = make_uint4(rh[0], rh[1], rh[2], rh[3]);
      *reinterpret_cast<uint4*>(arow + umma::sw128(row, 2 + half)) = make_uint4(ih[0], ih[1], ih[2], ih[3]);
      *reinterpret_cast<uint4*>(arow + umma::sw128(row, 4 + half)) = make_uint4(rl[0], rl[1], rl[2], rl[3]);
      *reinterpret_cast<uint4*>(arow + umma::sw128(row, 6 + half)) = make_uint4(il[0], il[1], il[2], il[3]);
    }
  }
  // the tensor core (async proxy) reads what the threads wrote; every thread
  // has also finished reading buf, which the outputs overwrite below
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  __syncthreads();
  if (t == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    constexpr uint32_t IDESC = umma::idesc_bf16(128, 32);
#pragma unroll
    for (int tile = 0; tile < NT; ++tile) {
      if (tile * 128 < NB) {
        const unsigned d = U.tmem + (unsigned)(tile * 32);
        const unsigned a0 = U.a + tile * kUmmaTileBytes;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) umma::mma_f16(d, umma::sdesc(a0 + kk * 32), umma::sdesc(U.bm + kk * 32), IDESC, kk);
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) umma::mma_f16(d, umma::sdesc(a0 + kk * 32), umma::sdesc(U.bl + kk * 32), IDESC, 1);
      }
    }
    umma::mma_commit(U.bar);
  }
  if (!umma::mbar_wait(U.bar, U.phase) && (t & 31) == 0 && U.err) atomicOr(U.err, 1);
  U.phase ^= 1u;
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  uint32_t v[32];
  {
    const unsigned ta = U.tmem + ((unsigned)((warp & 3) * 32) << 16) + (unsigned)((warp >> 2) * 32);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(ta)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
  }
  if (mine) {
    const int base = (j - k) * R + k;
#pragma unroll
    for (int m = 0; m < 16; ++m)
      buf[G::idx(l, base + m * NS)] = make_float2(__uint_as_float(v[m]), __uint_as_float(v[16 + m]));
  }
  // the next pass's MMAs overwrite TMEM and A: every warp's loads are done
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
}

// TCM: 0 SIMT butterflies, 1 radix-16 passes on mma.sync, 2 radix-16 passes on tcgen05
template <int N, int P, bool INV, int TCM>
__device__ __forceinline__ void fft_passes(float2* buf, const float2* tw, const DftFrag& F, UmmaFft* U,
                                           unsigned char* smem_base) {
  if constexpr (plan_radix(N, P) != 0) {
    if constexpr (TCM == 1 && plan_radix(N, P) == 16 && (Geom<N>::L * (N / 16)) % 8 == 0)
      fft_pass_tc16<N, P, INV>(buf, tw, F);
    else if constexpr (TCM == 2 && plan_radix(N, P) == 16) fft_pass_umma16<N, P, INV>(buf, tw, *U, smem_base);
    else fft_pass<N, P, INV>(buf, tw);
    fft_passes<N, P + 1, INV, TCM>(buf, tw, F, U, smem_base);
  }
}

// Transform all L lines in place.  Callers synchronise before the call (the
// lines must be fully written); the call ends with a barrier.  TCM selects the
// tensor-core radix-16 passes (1: mma.sync, 2: tcgen05 with the resources of *U).
template <int N, bool INV, int TCM = 0>
__device__ __forceinline__ void fft_lines(float2* buf, const float2* tw, UmmaFft* U = nullptr,
                                          unsigned char* smem_base = nullptr) {
  DftFrag F;
  if constexpr (TCM == 1) dft16_fragments<INV>(F);
  if constexpr (TCM == 2) {
    umma_dft16_b<INV, Geom<N>::T>(*U, smem_base);
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
  }
  fft_passes<N, 0, INV, TCM>(buf, tw, F, U, smem_base);
}

}  // namespace cdx
