// BF16 GEMM on the 5th-generation tensor cores (tcgen05 / UMMA, sm_103a):
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B K-major BF16, D FP32 row-major)
//
// CTA tile 128 x BN (BN = 64 or 128), K in steps of 64 (one 128-byte swizzle
// atom row).  128 threads stage A and B tiles with 16-byte cp.async into the
// canonical K-major SWIZZLE_128B layout (8-row x 128-byte atoms, 16-byte
// chunks XOR-swizzled by row % 8, atoms 1024 bytes apart); one thread issues
// the four m128nBNk16 MMAs of a stage with shared-memory descriptors, the
// accumulator lives in tensor memory (TMEM, BN FP32 columns), and
// tcgen05.commit arrives on the stage's mbarrier when the MMAs have read it.
// Each warp reads its 32 TMEM lanes (= 32 output rows) with tcgen05.ld.
//
// Every mbarrier wait is bounded: past the limit the CTA records an error in
// `err`, skips the remaining MMAs, waits (bounded) for what it issued, frees
// its TMEM and returns.  TMEM is freed on every path.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "cdx.h"
#include "cdx_host.h"
#include "cdx_unet.h"

namespace cdx {
namespace umma {

constexpr int BM = 128, BK = 64, ST = 3;
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

template <int BN>
__global__ void __launch_bounds__(128, 1) k_gemm_umma(const __nv_bfloat16* __restrict__ A,
                                                      const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                      int M, int N, int K, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-aligned stages: A (128 x 128 B), B (BN x 128 B)
  unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int A_BYTES = BM * 128, B_BYTES = BN * 128;
  unsigned char* sA = sm;
  unsigned char* sB = sm + ST * A_BYTES;
  __shared__ __align__(8) uint64_t bars[ST + 1];
  __shared__ unsigned tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int KT = (K + BK - 1) / BK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(BN)
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

  auto load = [&](int stage, int kt) {
    const int k0 = kt * BK;
    // A: 128 rows x 8 chunks = 1024 chunks, 8 per thread
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int q = tid + i * 128, r = q >> 3, c = q & 7;
      const int m = m0 + r, k = k0 + c * 8;
      const bool ok = m < M && k < K;
      cp16(smem_u32(sA + stage * A_BYTES) + sw128(r, c), ok ? (const void*)(A + (long long)m * K + k) : (const void*)A,
           ok);
    }
#pragma unroll
    for (int i = 0; i < BN * 8 / 128; ++i) {
      const int q = tid + i * 128, r = q >> 3, c = q & 7;
      const int n = n0 + r, k = k0 + c * 8;
      const bool ok = n < N && k < K;
      cp16(smem_u32(sB + stage * B_BYTES) + sw128(r, c), ok ? (const void*)(B + (long long)n * K + k) : (const void*)B,
           ok);
    }
  };

  constexpr uint32_t IDESC = idesc_bf16(BM, BN);
  bool failed = false;
  unsigned issued = 0;   // commits per stage barrier, to wait for them at the end
  unsigned uses[ST] = {0, 0, 0};
#pragma unroll
  for (int s = 0; s < ST - 1; ++s) {
    if (s < KT) load(s, s);
    cp_commit();
  }
  for (int kt = 0; kt < KT; ++kt) {
    const int s = kt % ST;
    cp_wait<ST - 2>();
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
      ++issued;
    }
    // before refilling stage (kt + ST - 1) % ST, the MMAs of step kt - 1 that read it must be done
    const int nk = kt + ST - 1;
    if (nk < KT) {
      const int ns = nk % ST;
      if (kt >= 1) {
        const unsigned par = uses[ns] & 1u;
        if (!failed && !mbar_wait(smem_u32(&bars[ns]), par)) failed = true;
        ++uses[ns];
      }
      load(ns, nk);
    }
    cp_commit();
  }
  cp_wait<0>();
  // the last MMAs: every step's commit is waited for in order (bounded)
  if (tid == 0 && !failed) {
    mma_commit(smem_u32(&bars[ST]));
  }
  __syncthreads();
  bool ok = !failed && (KT == 0 || mbar_wait(smem_u32(&bars[ST]), 0));
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
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
      if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (n0 + c0 + j < N) D[(long long)row * N + n0 + c0 + j] = __uint_as_float(v[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(BN) : "memory");
  (void)issued;
}

int smem_bytes(int bn) { return ST * (BM * 128 + bn * 128) + 1024; }

}  // namespace umma
}  // namespace cdx

using namespace cdx;

extern "C" int cdx_gemm_bf16_tc(const void* A, const void* B, float* D, int M, int N, int K, int* err_flag,
                                void* stream) {
  if (!A || !B || !D || !err_flag || M < 1 || N < 1 || K < 1) return set_error(CDX_ERR_ARG, "bad GEMM argument");
  if (K % 8) return set_error(CDX_ERR_ARG, "K must be a multiple of 8 (16-byte rows)");
  const int bn = N <= 64 ? 64 : 128;
  const int sm = umma::smem_bytes(bn);
  cudaError_t e;
  if (bn == 64) {
    e = cudaFuncSetAttribute(umma::k_gemm_umma<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
      umma::k_gemm_umma<64><<<dim3((M + 127) / 128, (N + 63) / 64), 128, sm, (cudaStream_t)stream>>>(
          (const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, M, N, K, err_flag);
  } else {
    e = cudaFuncSetAttribute(umma::k_gemm_umma<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e == cudaSuccess)
      umma::k_gemm_umma<128><<<dim3((M + 127) / 128, (N + 127) / 128), 128, sm, (cudaStream_t)stream>>>(
          (const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, M, N, K, err_flag);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("tensor-core GEMM: ") + cudaGetErrorString(e));
  return CDX_OK;
}
