// Per-length instantiation of the row/column pass kernels and their launchers.
// FP32 (tc == 0): the register-handoff kernels of cdx_rfft.cuh.  Tensor-core
// radix-16 passes: the staged kernels of cdx_kernels.cuh, on tcgen05 (tc == 1)
// or on warp-level mma.sync (tc == 2).
#pragma once
#include "cdx_rfft.cuh"

namespace cdx {

template <int N, int TCM>
cudaError_t prepare_tc_mode() {
  using G = Geom<N>;
  constexpr int X = TCM == 2 ? umma_smem_extra<N>() : 0;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(row_pass_kernel<N, ROW_FFT, TCM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES + X)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(row_pass_kernel<N, ROW_ITER, TCM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_ROW_ITER + X)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(col_pass_kernel<N, COL_FFT, TCM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES + X)) != cudaSuccess)
    return e;
  // at 4096 the noise-tolerant projection's three staged tiles and the tcgen05
  // operands exceed a CTA's 227 KB: that one combination is refused at launch
  constexpr int CI = G::SMEM_COL_CCD + X <= 232448 ? G::SMEM_COL_CCD + X : G::SMEM_COL_ITER + X;
  return cudaFuncSetAttribute(col_pass_kernel<N, COL_ITER, TCM>, cudaFuncAttributeMaxDynamicSharedMemorySize, CI);
}

template <int N>
cudaError_t prepare_tc() {
  cudaError_t e = prepare_tc_mode<N, 1>();
  return e != cudaSuccess ? e : prepare_tc_mode<N, 2>();
}

template <int N>
cudaError_t prepare_rk() {
  using G = Geom<N>;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(row_pass_rk<N, ROW_FFT, ALGO_ER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES)) != cudaSuccess)
    return e;
  const void* iter_kernels[] = {
      (const void*)row_pass_rk<N, ROW_ITER, ALGO_HIO>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_RAAR>,
      (const void*)row_pass_rk<N, ROW_ITER, ALGO_ER>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_POSER>,
      (const void*)row_pass_rk<N, ROW_ITER, ALGO_POSHIO>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_FHIO>};
  for (const void* k : iter_kernels)
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, RGeom<N>::SMEM_ROW_ITER)) !=
        cudaSuccess)
      return e;
  if constexpr (row_sq_ok<N>()) {
    const void* sq_kernels[] = {
        (const void*)row_pass_rk<N, ROW_ITER, ALGO_HIO, true>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_RAAR, true>,
        (const void*)row_pass_rk<N, ROW_ITER, ALGO_ER, true>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_POSER, true>,
        (const void*)row_pass_rk<N, ROW_ITER, ALGO_POSHIO, true>, (const void*)row_pass_rk<N, ROW_ITER, ALGO_FHIO, true>};
    for (const void* k : sq_kernels)
      if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, RGeom<N>::SMEM_ROW_ITER)) !=
          cudaSuccess)
        return e;
  }
  if ((e = cudaFuncSetAttribute(col_pass_rk<N, COL_FFT, PROJ_MODABS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_LINES)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(col_pass_rk<N, COL_ITER, PROJ_MODABS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                G::SMEM_COL_ITER)) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(col_pass_rk<N, COL_ITER, PROJ_CCD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              G::SMEM_COL_CCD);
}

// Raise the dynamic shared-memory limit of the kernels of length N on the
// current device (outside any stream capture).
template <int N>
cudaError_t prepare_len() {
  cudaError_t e = prepare_rk<N>();
  return e != cudaSuccess ? e : prepare_tc<N>();
}

// Programmatic dependent launch per length: measured on one GB300 it saves
// 1-2 % per iteration at 256^2 x64, 384^2 x16, 512^2 x16 and 1024^2 x4 and
// costs 1.3 % at 2048^2 (60.7 against 59.9 us), so that length launches plainly.
template <int N>
constexpr bool pass_pdl() { return N != 2048; }
// launch mode of a pass: the per-length default, or the autotuner's choice (1 plain, 2 PDL)
template <int N>
bool pdl_of(int mode) { return mode == 0 ? pass_pdl<N>() : mode == 2; }

template <int N>
cudaError_t launch_row(const RowArgs& a, int batch, cudaStream_t st) {
  using G = Geom<N>;
  dim3 grid((a.rows + G::L - 1) / G::L, batch);
  if (a.tc == 1) {   // tcgen05 (the kernels' TCM 2)
    constexpr int X = umma_smem_extra<N>();
    if (a.mode == ROW_ITER) row_pass_kernel<N, ROW_ITER, 2><<<grid, G::T, G::SMEM_ROW_ITER + X, st>>>(a);
    else row_pass_kernel<N, ROW_FFT, 2><<<grid, G::T, G::SMEM_LINES + X, st>>>(a);
  } else if (a.tc == 2) {   // mma.sync (the kernels' TCM 1)
    if (a.mode == ROW_ITER) row_pass_kernel<N, ROW_ITER, 1><<<grid, G::T, G::SMEM_ROW_ITER, st>>>(a);
    else row_pass_kernel<N, ROW_FFT, 1><<<grid, G::T, G::SMEM_LINES, st>>>(a);
  } else {
    constexpr int SM = RGeom<N>::SMEM_ROW_ITER;
    if (a.mode != ROW_ITER) return launch_pdl(row_pass_rk<N, ROW_FFT, ALGO_ER>, grid, G::T, G::SMEM_LINES, st, a, pdl_of<N>(a.pdl_mode));
    if constexpr (row_sq_ok<N>()) if (row_sq_layout<N>(a)) switch (a.algo) {   // the compile-time layout of square patterns
      case ALGO_HIO: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_HIO, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_RAAR: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_RAAR, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_ER: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_ER, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_POSER: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_POSER, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_POSHIO: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_POSHIO, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      default: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_FHIO, true>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
    }
    switch (a.algo) {   // unknown codes take the FHIO branch, as applySupport does (cdi.cc:25-36)
      case ALGO_HIO: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_HIO>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_RAAR: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_RAAR>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_ER: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_ER>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_POSER: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_POSER>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      case ALGO_POSHIO: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_POSHIO>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
      default: return launch_pdl(row_pass_rk<N, ROW_ITER, ALGO_FHIO>, grid, G::T, SM, st, a, pdl_of<N>(a.pdl_mode));
    }
  }
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_col(const ColArgs& a, int batch, cudaStream_t st) {
  using G = Geom<N>;
  dim3 grid((a.cols + G::L - 1) / G::L, batch);
  const int smem_iter = a.proj == PROJ_CCD ? G::SMEM_COL_CCD : G::SMEM_COL_ITER;
  if (a.tc == 1) {
    constexpr int X = umma_smem_extra<N>();
    if (a.mode == COL_ITER) col_pass_kernel<N, COL_ITER, 2><<<grid, G::T, smem_iter + X, st>>>(a);
    else col_pass_kernel<N, COL_FFT, 2><<<grid, G::T, G::SMEM_LINES + X, st>>>(a);
  } else if (a.tc == 2) {
    if (a.mode == COL_ITER) col_pass_kernel<N, COL_ITER, 1><<<grid, G::T, smem_iter, st>>>(a);
    else col_pass_kernel<N, COL_FFT, 1><<<grid, G::T, G::SMEM_LINES, st>>>(a);
  } else {
    if (a.mode != COL_ITER) return launch_pdl(col_pass_rk<N, COL_FFT, PROJ_MODABS>, grid, G::T, G::SMEM_LINES, st, a, pdl_of<N>(a.pdl_mode));
    if (a.proj == PROJ_CCD) return launch_pdl(col_pass_rk<N, COL_ITER, PROJ_CCD>, grid, G::T, smem_iter, st, a, pdl_of<N>(a.pdl_mode));
    return launch_pdl(col_pass_rk<N, COL_ITER, PROJ_MODABS>, grid, G::T, smem_iter, st, a, pdl_of<N>(a.pdl_mode));
  }
  return cudaGetLastError();
}

#define CDX_INSTANTIATE(N)                                                   \
  template cudaError_t prepare_len<N>();                                     \
  template cudaError_t launch_row<N>(const RowArgs&, int, cudaStream_t);     \
  template cudaError_t launch_col<N>(const ColArgs&, int, cudaStream_t);

}  // namespace cdx
