// Zernike pupil fit of the ptychographic probe phase (cdx_pty_zernike.cu).
#pragma once
#include <cuda_runtime.h>

namespace cdx {

constexpr int kZkMaxN = 40;                                   // util/ptycho.cpp:439
constexpr int kZkModes = (kZkMaxN + 1) * (kZkMaxN + 2) / 2;   // 861

// CTAs of the projection of a pd x pd crop (rows of its partial-coefficient buffer)
int zk_blocks(int pd);
// per-pixel table of the crop (pd * pd float4): coverage weight, centroid radius / (pd/2), angle, rebuilt flag
cudaError_t zk_table(float4* tab, int pd, cudaStream_t st);
// project the centred pd x pd crop of P on the basis, threshold, write the rebuilt crop padded with zeros into P
cudaError_t zk_fit(float2* P, int rows, int cols, int pd, const float4* tab, float2* part, float2* coef,
                   cudaStream_t st);

}  // namespace cdx
