// Launchers of the auxiliary CDI kernels (cdx_misc.cu).
#pragma once
#include "cdx_types.h"

namespace cdx {

cudaError_t amp_from_pattern(const float* inten, float* amp, long long n, cudaStream_t st);
cudaError_t scale_complex(float2* x, float s, long long n, cudaStream_t st);
cudaError_t scale_real(float* x, float s, long long n, cudaStream_t st);
cudaError_t convert_fo_real(const float* in, float* out, int rows, int cols, int batch, cudaStream_t st);
cudaError_t convert_fo_complex(const float2* in, float2* out, int rows, int cols, int batch, cudaStream_t st);
cudaError_t to_tiled(const float* in, float* out, int rows, int cols, int tl, long long out_stride, int batch,
                     cudaStream_t st);
cudaError_t mod_abs(float2* psi, const float* inten, long long n, cudaStream_t st);
cudaError_t mod_ccd(float2* psi, const float* inten, const float* bs, int noise, float scale, float rcolor,
                    long long n, cudaStream_t st);
cudaError_t apply_support(float2* rho, const float2* rhop, const float* spt, float thr, float beta, int algo,
                          long long n, cudaStream_t st);
cudaError_t rect_support(float* spt, int rows, int cols, int batch, int sx, int sy, int ex, int ey, cudaStream_t st);
cudaError_t support_bits(const float* spt, const PatState* st_or_null, float fixed_thr, uint32_t* bits, int rows,
                         int cols, int batch, cudaStream_t st);
// Kernel attributes of the stencil kernels (once per device, outside capture).
cudaError_t misc_prepare();
cudaError_t shrinkwrap(const float2* rho, float2* tmp, float* spt, const float* wx, int radx, const float* wy,
                       int rady, int rows, int cols, int batch, int mod2_first, float s, float* pmax, double* psum,
                       int nblk, PatState* stt, double shrink_threshold, cudaStream_t st);
cudaError_t pattern_amp_sum(const float* amp, long long npx, int batch, double* part, int nblk, PatState* stt,
                            cudaStream_t st);
// The residual and the R-factor of the final Psi in one pass (2 * nblk partials per pattern;
// the R-factor divides by the pattern's amp_sum).
cudaError_t residual_rfactor(const float2* psi, const float* inten, long long npx, int batch, double* part, int nblk,
                             PatState* stt, cudaStream_t st);
cudaError_t rfactor_from_partials(const double* part, int nblk, int batch, PatState* stt, double stop, int iter,
                                  int plateau, float tol, cudaStream_t st);
cudaError_t run_begin(PatState* stt, int batch, cudaStream_t st);
cudaError_t state_init(PatState* stt, int batch, float thr, cudaStream_t st);
cudaError_t random_start(const float* inten, const float* bs, float bs_thr, float2* psi, long long npx, int batch,
                         unsigned long long seed, cudaStream_t st);

// PRTF (src/post_gpu/cdi.cc:355-380, 424-440): one step's ER-correlation and
// phase, the phasor accumulation, and the polar sums of cart2polar_kernel +
// edgeReduce (src/gpu/cudaConfig.cu:1027-1063).
cudaError_t prtf_step(const float2* rhop, const uint32_t* bits, int rows, int cols, int batch, float2* cache,
                      float2* gamma0, int first, double* part, int nblk, PrtfState* ps, const PatState* stt,
                      cudaStream_t st);
cudaError_t prtf_accum(const float2* psi_proj, float2* map, float* mask_or_null, long long npx, int batch,
                       const PrtfState* ps, const PatState* stt, cudaStream_t st);
cudaError_t prtf_polar(const float* mask, const float2* map, float inv_count, int rows, int cols, int batch,
                       float* out, cudaStream_t st);
}  // namespace cdx
