// Per-length instantiation of the row/column pass kernels and their launchers.
#pragma once
#include "cdx_kernels.cuh"

namespace cdx {

template <int N, bool TC>
cudaError_t prepare_variant() {
  using G = Geom<N>;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(row_pass_kernel<N, ROW_FFT, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(row_pass_kernel<N, ROW_ITER, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_ROW_ITER)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(col_pass_kernel<N, COL_FFT, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES)) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(col_pass_kernel<N, COL_ITER, TC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              G::SMEM_COL_CCD);
}

// Raise the dynamic shared-memory limit of the kernels of length N on the
// current device (outside any stream capture).
template <int N>
cudaError_t prepare_len() {
  cudaError_t e = prepare_variant<N, false>();
  return e != cudaSuccess ? e : prepare_variant<N, true>();
}

template <int N, bool TC>
void launch_row_variant(const RowArgs& a, dim3 grid, cudaStream_t st) {
  using G = Geom<N>;
  if (a.mode == ROW_ITER) row_pass_kernel<N, ROW_ITER, TC><<<grid, G::T, G::SMEM_ROW_ITER, st>>>(a);
  else row_pass_kernel<N, ROW_FFT, TC><<<grid, G::T, G::SMEM_LINES, st>>>(a);
}

template <int N, bool TC>
void launch_col_variant(const ColArgs& a, dim3 grid, cudaStream_t st) {
  using G = Geom<N>;
  if (a.mode == COL_ITER)
    col_pass_kernel<N, COL_ITER, TC><<<grid, G::T, a.proj == PROJ_CCD ? G::SMEM_COL_CCD : G::SMEM_COL_ITER, st>>>(a);
  else col_pass_kernel<N, COL_FFT, TC><<<grid, G::T, G::SMEM_LINES, st>>>(a);
}

template <int N>
cudaError_t launch_row(const RowArgs& a, int batch, cudaStream_t st) {
  using G = Geom<N>;
  dim3 grid((a.rows + G::L - 1) / G::L, batch);
  if (a.tc) launch_row_variant<N, true>(a, grid, st);
  else launch_row_variant<N, false>(a, grid, st);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_col(const ColArgs& a, int batch, cudaStream_t st) {
  using G = Geom<N>;
  dim3 grid((a.cols + G::L - 1) / G::L, batch);
  if (a.tc) launch_col_variant<N, true>(a, grid, st);
  else launch_col_variant<N, false>(a, grid, st);
  return cudaGetLastError();
}

#define CDX_INSTANTIATE(N)                                                   \
  template cudaError_t prepare_len<N>();                                     \
  template cudaError_t launch_row<N>(const RowArgs&, int, cudaStream_t);     \
  template cudaError_t launch_col<N>(const ColArgs&, int, cudaStream_t);

}  // namespace cdx
