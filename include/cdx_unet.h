/* Learned warm start for the CDI iteration: a U-Net trained on the GPU by
 * hand-written CUDA kernels (cdixx_gb300/csrc/cdx_unet*.cu).
 *
 * No reference counterpart on the phase-retrieval path: the reference's
 * U-Nets (python/UNet.py:45-85, trained by python/train.py:17-29 with Adam and
 * MSE) are PyTorch scripts for pattern clean-up; this network follows their
 * building blocks (3x3 conv, normalisation, LeakyReLU, stride-2 conv down,
 * transposed conv up, concatenated skips) and maps a diffraction pattern to an
 * initial object for HIO/RAAR.
 *
 * Network: input log(1 + I) / max log(1 + I), centred, one channel (padded to
 * 8); `levels` resolutions with base * 2^l channels; every convolution is
 * followed by GroupNorm (`groups`) and LeakyReLU (`slope`); a 1x1 head gives
 * four channels in the centred object frame: amplitude, cos(phase),
 * sin(phase), support logit.  Weights are kept in FP32 (Adam) with BF16
 * copies for the tensor-core products; accumulation is FP32.
 *
 * Loss per pattern (mean over pixels), minimum over the object and its twin
 * conj(rho(-r)) (|FFT|^2 cannot tell them apart):
 *   (a - a_t)^2 + a_t ((c - cos p_t)^2 + (s - sin p_t)^2) + w_s BCE(logit, s_t),
 * averaged over the patterns of the batch.
 *
 * All array arguments are device pointers; sizes are in elements.
 */
#ifndef CDX_UNET_H
#define CDX_UNET_H

#ifdef __cplusplus
extern "C" {
#endif

#pragma GCC visibility push(default)

typedef struct cdx_unet cdx_unet;

typedef struct {
  int n;              /* pattern side (a multiple of 2^(levels-1) and of 8) */
  int levels;         /* resolutions (>= 2) */
  int base;           /* channels at full resolution (a multiple of 8) */
  int batch;          /* largest batch a call may pass */
  int groups;         /* GroupNorm groups (divides base) */
  float slope;        /* LeakyReLU negative slope */
  float support_weight; /* w_s */
  unsigned long long seed; /* weight initialisation */
  int umma;           /* 1: forward and data-gradient convolutions on tcgen05/TMEM; 0 (default):
                         warp-level mma.sync, faster for these channel counts (the weight gradient
                         is mma.sync in both; the two give the same bits) */
} cdx_unet_config;

int cdx_unet_config_default(cdx_unet_config* c);
int cdx_unet_create(const cdx_unet_config* c, void* stream, cdx_unet** out);
void cdx_unet_destroy(cdx_unet* u);
long long cdx_unet_param_count(const cdx_unet* u);
/* FP32 parameters / last gradients in the documented flat order, host memory */
int cdx_unet_get_params(const cdx_unet* u, float* host, long long count);
int cdx_unet_set_params(cdx_unet* u, const float* host, long long count);
int cdx_unet_get_grads(const cdx_unet* u, float* host, long long count);

/* out[b][4][n][n] (centred) from intensity[b][n][n] (FFT order), b < count */
int cdx_unet_forward(cdx_unet* u, const float* intensity, float* out, int count);
/* forward + loss + backward (gradients kept in the network); *loss = the batch loss */
int cdx_unet_loss_backward(cdx_unet* u, const float* intensity, const float* amp_t, const float* phase_t,
                           const float* support_t, int count, double* loss);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the last gradients */
int cdx_unet_adam_step(cdx_unet* u, float lr);
/* Warm start for the iteration from the network output of cdx_unet_forward:
 * rho0 = a e^{i atan2(s, c)} on sigmoid(logit) > 0.5 (the object frame: the
 * object centred in the array, as the reference keeps objectWave), then
 * psi0[b] = sqrt(I) e^{i arg FFT(rho0)} (complex64, the pattern's FFT order)
 * and support[b] = the mask dilated by `dilate` pixels (float 0/1, object frame). */
int cdx_unet_warm_start(cdx_unet* u, const float* intensity, const float* out, int count, int dilate, void* psi0,
                        float* support);

/* Seeded synthetic training pairs on the GPU (forward model: blob objects,
 * I = |FFT(rho)|^2 scaled to `photons` and Poisson-sampled).  Pattern p of
 * the call uses counter-based random numbers keyed by (seed, first + p).
 * intensity [count][n][n] FFT order; amp_t, phase_t, support_t centred (any
 * of the three may be null).  photons < 0: no Poisson step, I scaled to -photons.
 * The work is queued on `stream` and the call returns without waiting for it:
 * a consumer on another stream must wait for `stream` first. */
int cdx_forward_model(int n, int count, unsigned long long seed, long long first, double photons,
                      float* intensity, float* amp_t, float* phase_t, float* support_t, void* stream);

/* D[m][n] = sum_k A[m][k] B[n][k] on the tcgen05 tensor cores (A, B K-major
 * BF16 device arrays, D FP32 row-major; K a multiple of 8).  *err_flag (device
 * int, set by the caller to 0) becomes 1 if a tile's pipeline wait timed out. */
int cdx_gemm_bf16_tc(const void* A, const void* B, float* D, int M, int N, int K, int* err_flag, void* stream);

#pragma GCC visibility pop

#ifdef __cplusplus
}
#endif
#endif
