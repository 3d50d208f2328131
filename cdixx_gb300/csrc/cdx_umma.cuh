// BF16 GEMM core on the 5th-generation tensor cores (tcgen05 / UMMA, sm_103a):
//     D[m][n] = sum_k A[m][k] * B[n][k]      (A, B BF16 read K-major, FP32 accumulate)
//
// CTA tile 128 x BN (BN = 32, 64 or 128), K in steps of 64 (one 128-byte
// swizzle atom row), operands staged with 16-byte cp.async into the
// canonical K-major SWIZZLE_128B layout (8-row x 128-byte atoms, 16-byte
// chunks XOR-swizzled by row % 8, atoms 1024 bytes apart), MMAs issued by one
// thread with shared-memory descriptors, accumulator in tensor memory (TMEM)
// read back with tcgen05.ld.  The kernel (k_umma_ps) is persistent and warp
// specialised: producer warps, an MMA warp and epilogue warps synchronised by
// mbarriers, a multi-stage operand pipeline and a double-buffered accumulator.
//
// Where the operands come from and where results go is a policy (Op):
//   Op::Row  row(m)           per output row, computed once per tile
//   Op::Kc   kc(k)            per K chunk (8 consecutive k), once per stage
//   a_src(Row, Kc) / b_src(n, k): source of 8 BF16 (16 bytes), or null (zero)
//   store(m, n0, v[16], count): results v[j] of columns n0 + j, j < count
//
// Every mbarrier wait is bounded: past the limit the CTA records an error in
// `err`, stops issuing, drains what it started and frees its TMEM.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "cdx_types.h"

namespace cdx {
namespace umma {

constexpr int BM = 128, BK = 64;
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

// ---------------------------------------------------------------- pipeline shape
constexpr int WS_ST = 4;      // operand stages
constexpr int WS_D = 2;       // K steps of copies a producer keeps in flight beyond the one it signals:
                              // for step g it waits for its copies of step g - WS_D, fences them for
                              // the tensor core and arrives on that stage's `full` barrier
inline int ws_smem_bytes(int bn) { return WS_ST * (BM * 128 + bn * 128) + 1024; }

__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(bar) : "memory");
}

// ---------------------------------------------------------------- persistent
// A CTA loops over the M tiles blockIdx.x,
// blockIdx.x + gridDim.x, ... of its N tile, so the copy pipeline runs
// without a break from one tile into the next, and the accumulator is double
// buffered in TMEM (2 x BN columns) so the epilogue of tile i overlaps the
// MMAs of tile i + 1.  Roles (288 threads):
//   warps 0-3  producers: cp.async stages, `full` after the copies landed;
//   warps 4-7  epilogue: wait `tfull[b]`, tcgen05.ld (warp w: lanes 32 (w-4)..),
//              store, release the buffer with `tempty[b]` (128 arrivals);
//   warp 8     one lane issues the MMAs: waits `tempty[b]` before a tile, `full`
//              before a K step, commits each step to `empty` and each tile to
//              `tfull[b]`; the warp allocates and frees the TMEM.
// Every wait is bounded; a role that gives up sets *err and the shared abort
// flag, which ends every other role's waits at once.
constexpr int PS_THREADS = 288;

__device__ __forceinline__ bool mbar_wait_or_abort(unsigned bar, unsigned parity, volatile int* abort_flag) {
  for (unsigned i = 0; i < kSpinLimit; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 63) == 63 && *abort_flag) return false;
  }
  return false;
}

template <int BN, class Op>
__global__ void __launch_bounds__(PS_THREADS, 1) k_umma_ps(Op op, int M, int N, int K, int* __restrict__ err) {
  static_assert(BN == 32 || BN == 64 || BN == 128, "UMMA N tile");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  constexpr int A_BYTES = BM * 128, B_BYTES = BN * 128;
  unsigned char* sA = sm;
  unsigned char* sB = sm + WS_ST * A_BYTES;
  __shared__ __align__(8) uint64_t full[WS_ST], empty[WS_ST], tfull[2], tempty[2], done;
  __shared__ unsigned tmem_base;
  __shared__ volatile int abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int n0 = blockIdx.y * BN;
  const int KT = (K + BK - 1) / BK;
  const int MT = (M + BM - 1) / BM;
  constexpr int TC = 2 * BN < 32 ? 32 : 2 * BN;   // two accumulators

  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < WS_ST; ++i) {
      mbar_init(smem_u32(&full[i]), 128);
      mbar_init(smem_u32(&empty[i]), 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(smem_u32(&tfull[i]), 1);
      mbar_init(smem_u32(&tempty[i]), 128);
    }
    mbar_init(smem_u32(&done), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = tmem_base;
  auto give_up = [&]() {
    abort_flag = 1;
    atomicExch(err, 1);
  };

  if (warp < 4) {
    // ------------------------------------------------------------ producers
    const int cch = tid & 7, r0 = tid >> 3;
    long long g = 0;   // K steps issued by this thread, over all its tiles
    bool failed = false;
    for (int tile = blockIdx.x; tile < MT && !failed; tile += gridDim.x) {
      const int m0 = tile * BM;
      typename Op::Row rows[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) rows[i] = op.row(m0 + r0 + 16 * i, M);
      for (int kt = 0; kt < KT; ++kt) {
        const int s = (int)(g % WS_ST);
        const long long use = g / WS_ST;
        if (use > 0 && !mbar_wait_or_abort(smem_u32(&empty[s]), (unsigned)((use - 1) & 1), &abort_flag)) {
          failed = true;
          break;
        }
        const int k = kt * BK + cch * 8;
        const typename Op::Kc kc = op.kc(k, K);
        const unsigned a_base = smem_u32(sA + s * A_BYTES), b_base = smem_u32(sB + s * B_BYTES);
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
        cp_commit();
        if (g >= WS_D) {
          cp_wait<WS_D>();
          asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
          mbar_arrive(smem_u32(&full[(g - WS_D) % WS_ST]));
        }
        ++g;
      }
    }
    cp_wait<0>();
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    if (failed) {
      if ((tid & 31) == 0) give_up();
    } else {
      for (long long q = g > WS_D ? g - WS_D : 0; q < g; ++q) mbar_arrive(smem_u32(&full[q % WS_ST]));
    }
  } else if (warp < 8) {
    // ------------------------------------------------------------ epilogue
    const int ew = warp - 4, lane = tid & 31;
    int t = 0;
    for (int tile = blockIdx.x; tile < MT; tile += gridDim.x, ++t) {
      const int b = t & 1;
      if (!mbar_wait_or_abort(smem_u32(&tfull[b]), (unsigned)((t >> 1) & 1), &abort_flag)) {
        if (lane == 0) give_up();
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const int row = tile * BM + ew * 32 + lane;
#pragma unroll
      for (int c0 = 0; c0 < BN; c0 += 16) {
        uint32_t v[16];
        const unsigned ta = tmem + ((unsigned)(ew * 32) << 16) + (unsigned)(b * BN + c0);
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
      asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
      mbar_arrive(smem_u32(&tempty[b]));
    }
  } else {
    // ------------------------------------------------------------ MMA lane
    if ((tid & 31) == 0) {
      constexpr uint32_t IDESC = idesc_bf16(BM, BN);
      long long g = 0;
      int t = 0;
      bool failed = false;
      for (int tile = blockIdx.x; tile < MT && !failed; tile += gridDim.x, ++t) {
        const int b = t & 1;
        if (t >= 2 && !mbar_wait_or_abort(smem_u32(&tempty[b]), (unsigned)(((t >> 1) - 1) & 1), &abort_flag)) {
          failed = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const unsigned d = tmem + (unsigned)(b * BN);
        for (int kt = 0; kt < KT; ++kt, ++g) {
          const int s = (int)(g % WS_ST);
          if (!mbar_wait_or_abort(smem_u32(&full[s]), (unsigned)((g / WS_ST) & 1), &abort_flag)) {
            failed = true;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const unsigned a0 = smem_u32(sA + s * A_BYTES), b0 = smem_u32(sB + s * B_BYTES);
#pragma unroll
          for (int kk = 0; kk < BK / 16; ++kk)
            mma_f16(d, sdesc(a0 + kk * 32), sdesc(b0 + kk * 32), IDESC, (kt > 0 || kk > 0) ? 1 : 0);
          mma_commit(smem_u32(&empty[s]));
        }
        if (!failed) mma_commit(smem_u32(&tfull[b]));
      }
      if (failed) give_up();
      mma_commit(smem_u32(&done));   // arrives when every MMA this lane issued is complete
    }
    __syncwarp();
  }
  // TMEM is freed after the last MMA has completed and the epilogue's reads are done
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 8) {
    if (!mbar_wait(smem_u32(&done), 0) && (tid & 31) == 0) atomicExch(err, 1);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TC) : "memory");
  }
}

inline int ps_smem_bytes(int bn) { return ws_smem_bytes(bn); }

// Launch k_umma_ps with as many CTAs per N tile as fit on the device at once
// (each loops over M tiles).  The attribute and occupancy are looked up once
// per instantiation and device (a benign race between host threads writes
// the same value).
template <int BN, class Op>
cudaError_t launch_ps(const Op& op, int M, int N, int K, int* err, cudaStream_t st) {
  static int cached[64];   // resident CTAs per SM, per device (0: not looked up yet)
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int per_sm = (dev >= 0 && dev < 64) ? cached[dev] : 0;
  if (per_sm == 0) {
    if ((e = cudaFuncSetAttribute(k_umma_ps<BN, Op>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  ps_smem_bytes(BN))) != cudaSuccess)
      return e;
    int b = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_umma_ps<BN, Op>, PS_THREADS, ps_smem_bytes(BN))) !=
        cudaSuccess)
      return e;
    per_sm = b > 0 ? b : 1;
    if (dev >= 0 && dev < 64) cached[dev] = per_sm;
  }
  const int mt = (M + BM - 1) / BM, nt = (N + BN - 1) / BN;
  const long long slots = (long long)per_sm * sm_count();
  const int gx = (int)std::max(1LL, std::min<long long>(mt, slots / nt > 0 ? slots / nt : 1));
  k_umma_ps<BN, Op><<<dim3(gx, nt), PS_THREADS, ps_smem_bytes(BN), st>>>(op, M, N, K, err);
  return cudaGetLastError();
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
