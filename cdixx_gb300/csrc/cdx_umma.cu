// C ABI of the tcgen05 BF16 GEMM (cdx_umma.cuh): D = A B^T with dense
// K-major BF16 operands.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "cdx.h"
#include "cdx_host.h"
#include "cdx_unet.h"
#include "cdx_umma.cuh"

using namespace cdx;

extern "C" int cdx_gemm_bf16_tc(const void* A, const void* B, float* D, int M, int N, int K, int* err_flag,
                                void* stream) {
  if (!A || !B || !D || !err_flag || M < 1 || N < 1 || K < 1) return set_error(CDX_ERR_ARG, "bad GEMM argument");
  if (K % 8) return set_error(CDX_ERR_ARG, "K must be a multiple of 8 (16-byte rows)");
  umma::DenseOp op{(const __nv_bfloat16*)A, (const __nv_bfloat16*)B, D, K, N};
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (N <= 32) e = umma::launch_ps<32>(op, M, N, K, err_flag, st);
  else if (N <= 64) e = umma::launch_ps<64>(op, M, N, K, err_flag, st);
  else e = umma::launch_ps<128>(op, M, N, K, err_flag, st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("tensor-core GEMM: ") + cudaGetErrorString(e));
  return CDX_OK;
}
