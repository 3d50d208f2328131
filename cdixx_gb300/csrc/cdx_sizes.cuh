// Per-length instantiation of the row/column pass kernels and their launchers.
#pragma once
#include "cdx_kernels.cuh"

namespace cdx {

// Raise the dynamic shared-memory limit of both kernels of length N on the
// current device (outside any stream capture).
template <int N>
cudaError_t prepare_len() {
  constexpr int SM = Geom<N>::SMEM;
  cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(col_pass_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, SM);
}

template <int N>
cudaError_t launch_row(const RowArgs& a, int batch, cudaStream_t st) {
  constexpr int L = Geom<N>::L, T = Geom<N>::T, SM = Geom<N>::SMEM;
  dim3 grid((a.rows + L - 1) / L, batch);
  row_pass_kernel<N><<<grid, T, SM, st>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_col(const ColArgs& a, int batch, cudaStream_t st) {
  constexpr int L = Geom<N>::L, T = Geom<N>::T, SM = Geom<N>::SMEM;
  dim3 grid((a.cols + L - 1) / L, batch);
  col_pass_kernel<N><<<grid, T, SM, st>>>(a);
  return cudaGetLastError();
}

#define CDX_INSTANTIATE(N)                                                   \
  template cudaError_t prepare_len<N>();                                     \
  template cudaError_t launch_row<N>(const RowArgs&, int, cudaStream_t);     \
  template cudaError_t launch_col<N>(const ColArgs&, int, cudaStream_t);

// The supported lengths: 2^a 3^b from 16 to 4096.
#define CDX_FOR_EACH_SIZE(X) \
  X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256) X(384) X(512) X(768) X(1024) \
  X(1536) X(2048) X(3072) X(4096)

}  // namespace cdx
