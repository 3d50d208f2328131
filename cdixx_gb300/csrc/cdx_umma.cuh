// BF16 GEMM core on the 5th-generation tensor cores (tcgen05 / UMMA, sm_103a):
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B BF16 read K-major, FP32 accumulate)
//
// CTA tile 128 x BN (BN = 32, 64 or 128), K in steps of 64 (one 128-byte
// swizzle atom row).  128 threads stage A and B tiles with 16-byte cp.async
// into the canonical K-major SWIZZLE_128B layout (8-row x 128-byte atoms,
// 16-byte chunks XOR-swizzled by row % 8, atoms 1024 bytes apart); one thread
// issues the four m128nBNk16 MMAs of a stage with shared-memory descriptors,
// the accumulator lives in tensor memory (TMEM, BN FP32 columns), and
// tcgen05.commit arrives on the stage's mbarrier when the MMAs have read it.
// Each warp reads its 32 TMEM lanes (= 32 output rows) with tcgen05.ld.
//
// Where the operands come from and where results go is a policy (Op):
//   Op::Row  row(m)           per output row, computed once per kernel
//   Op::Kc   kc(k)            per K chunk (8 consecutive k), once per stage
//   a_src(Row, Kc) / b_src(n, k): source of 8 BF16 (16 bytes), or null (zero)
//   store(m, n0, v[16], count): results v[j] of columns n0 + j, j < count
//
// Every mbarrier wait is bounded: past the limit the CTA records an error in
// `err`, skips the remaining MMAs, frees its TMEM and returns.  TMEM is freed
// on every path.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace cdx {
namespace umma {

constexpr int BM = 128, BK = 64, ST = 3;
// stages loaded ahead: a refill waits on the MMAs of the previous step (a fourth
// stage with a refill two steps back was slower: fewer CTAs per SM)
constexpr int PF = ST - 1;
constexpr unsigned kSpinLimit = 1u << 22;   // mbarrier polls before giving up

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void cp16(unsigned dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// true when the phase with parity `parity` has completed
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (unsigned i = 0; i < kSpinLimit; ++i)
    if (mbar_try(bar, parity)) return true;
  return false;
}

// shared-memory matrix descriptor, K-major SWIZZLE_128B: start >> 4 (bits 0-13),
// leading byte offset (unused for this layout, 1), stride byte offset 1024 >> 4
// (bits 32-45), descriptor version 1 (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63)
__device__ __forceinline__ uint64_t sdesc(unsigned saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits
// 7-9, 10-12 = 1), both K-major, N >> 3 (bits 17-22), M >> 4 (bits 24-28)
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(unsigned tmem, uint64_t a, uint64_t b, uint32_t idesc, int accum) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void mma_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(bar) : "memory");
}

// byte offset of 16-byte chunk c (0..7) of row r in a SWIZZLE_128B K-major tile
__device__ __forceinline__ unsigned sw128(int r, int c) {
  return (unsigned)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

inline int smem_bytes(int bn) { return ST * (BM * 128 + bn * 128) + 1024; }

template <int BN, class Op>
__global__ void __launch_bounds__(128, 1) k_umma(Op op, int M, int N, int K, int* __restrict__ err) {
  static_assert(BN == 32 || BN == 64 || BN == 128, "UMMA N tile");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int A_BYTES = BM * 128, B_BYTES = BN * 128;
  unsigned char* sA = sm;
  unsigned char* sB = sm + ST * A_BYTES;
  __shared__ __align__(8) uint64_t bars[ST + 1];
  __shared__ unsigned tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int KT = (K + BK - 1) / BK;
  constexpr int TC = BN < 32 ? 32 : BN;   // TMEM columns (a power of two >= 32)

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i <= ST; ++i) mbar_init(smem_u32(&bars[i]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = tmem_base;

  // this thread stages chunk c = tid & 7 of rows (tid >> 3) + 16 i of both tiles
  const int cch = tid & 7, r0 = tid >> 3;
  typename Op::Row rows[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) rows[i] = op.row(m0 + r0 + 16 * i, M);

  auto load = [&](int stage, int kt) {
    const int k = kt * BK + cch * 8;
    const typename Op::Kc kc = op.kc(k, K);
    const unsigned a_base = smem_u32(sA + stage * A_BYTES), b_base = smem_u32(sB + stage * B_BYTES);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const __nv_bfloat16* src = op.a_src(rows[i], kc);
      cp16(a_base + sw128(r0 + 16 * i, cch), src ? (const void*)src : op.dummy(), src != nullptr);
    }
#pragma unroll
    for (int i = 0; i < BN / 16; ++i) {
      const int n = n0 + r0 + 16 * i;
      const __nv_bfloat16* src = (n < N && k < K) ? op.b_src(n, k) : nullptr;
      cp16(b_base + sw128(r0 + 16 * i, cch), src ? (const void*)src : op.dummy(), src != nullptr);
    }
  };

  constexpr uint32_t IDESC = idesc_bf16(BM, BN);
  bool failed = false;
  unsigned uses[ST] = {0, 0, 0};
#pragma unroll
  for (int s = 0; s < PF; ++s) {
    if (s < KT) load(s, s);
    cp_commit();
  }
  for (int kt = 0; kt < KT; ++kt) {
    const int s = kt % ST;
    cp_wait<PF - 1>();
    // the async proxy (tensor core) reads what the generic proxy wrote
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (tid == 0 && !failed) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned a0 = smem_u32(sA + s * A_BYTES), b0 = smem_u32(sB + s * B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk)   // 16 BF16 = 32 bytes along K inside the swizzle atom
        mma_f16(tmem, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), IDESC, (kt > 0 || kk > 0) ? 1 : 0);
      mma_commit(smem_u32(&bars[s]));
    }
    // before refilling stage (kt + PF) % ST, the MMAs of step kt + PF - ST that read it must be done
    const int nk = kt + PF;
    if (nk < KT) {
      const int ns = nk % ST;
      if (nk >= ST) {
        const unsigned par = uses[ns] & 1u;
        if (!failed && !mbar_wait(smem_u32(&bars[ns]), par)) failed = true;
        ++uses[ns];
      }
      load(ns, nk);
    }
    cp_commit();
  }
  cp_wait<0>();
  if (tid == 0 && !failed) mma_commit(smem_u32(&bars[ST]));   // arrives when every MMA of the CTA is done
  __syncthreads();
  const bool ok = !failed && (KT == 0 || mbar_wait(smem_u32(&bars[ST]), 0));
  if (!ok && (tid & 31) == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (ok && KT > 0) {
    // warp w reads TMEM lanes 32w..32w+31 (rows m0 + 32w + lane), 16 columns at a time
    const int row = m0 + warp * 32 + (tid & 31);
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 16) {
      uint32_t v[16];
      const unsigned ta = tmem + ((unsigned)(warp * 32) << 16) + (unsigned)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(ta)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M && n0 + c0 < N) {
        float f[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) f[j] = __uint_as_float(v[j]);
        op.store(row, n0 + c0, f, min(16, N - n0 - c0));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC) : "memory");
}

// Dense operands: A [M][K], B [N][K] (K-major BF16), D [M][N] FP32.
struct DenseOp {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  float* D;
  int K, N;
  struct Row { const __nv_bfloat16* p; };
  struct Kc { int k; bool ok; };
  __device__ Row row(int m, int M) const { return Row{m < M ? A + (long long)m * K : nullptr}; }
  __device__ Kc kc(int k, int K_) const { return Kc{k, k < K_}; }
  __device__ const __nv_bfloat16* a_src(const Row& r, const Kc& c) const { return (r.p && c.ok) ? r.p + c.k : nullptr; }
  __device__ const __nv_bfloat16* b_src(int n, int k) const { return B + (long long)n * K + k; }
  __device__ const void* dummy() const { return A; }
  __device__ void store(int m, int n0, const float* v, int cnt) const {
    for (int j = 0; j < cnt; ++j) D[(long long)m * N + n0 + j] = v[j];
  }
};

}  // namespace umma
}  // namespace cdx
