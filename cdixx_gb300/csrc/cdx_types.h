// Kernel argument blocks and codes shared by the CUDA translation units.
//
// HBM layouts.  A rows x cols array is either row-major (element (r,c) at
// r*cols + c) or column-tiled with tile width TW (a power of two): element
// (r,c) at ((c/TW)*rows + r)*TW + c%TW, the width padded to a multiple of TW.
// A column-pass CTA covering TW columns then reads one contiguous block, and
// a row-pass CTA covering several rows moves whole 32-byte sectors.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cdx {

// Update codes: the reference's Algorithm enum (include/format.hpp:22).
enum : int {
  ALGO_RAAR = 0, ALGO_ER = 1, ALGO_POSER = 2, ALGO_HIO = 3, ALGO_POSHIO = 4, ALGO_FHIO = 5,
  ALGO_SHRINKWRAP = 6, ALGO_XCORRELATION = 7, ALGO_KKT = 8, ALGO_TV = 9, ALGO_CNT = 10
};

enum : int { ROW_FFT = 0, ROW_ITER = 1 };
enum : int { COL_FFT = 0, COL_ITER = 1 };
enum : int { PROJ_MODABS = 0, PROJ_CCD = 1 };

// Per-pattern device state of the shrinkwrap (the reference keeps it in host
// locals of phaseRetrieve and in __constant__ vars.threshold).
struct PatState {
  float threshold;   // vars.threshold
  float avg;         // avg of phaseRetrieve (0 until the first shrinkwrap)
  float maxv;        // last max of the blurred support
  float sum;         // last sum of the blurred support
  double rfactor;    // last R-factor
  double amp_sum;    // sum sqrt(I)
  double residual;   // final residual
  int flags;         // bit 0: NaN/zero max seen at a shrinkwrap; bit 1: R <= stop reached (or a
                     // plateau); bit 2: frozen (set by the column pass after bit 1; both passes then
                     // skip); bit 3: the plateau set bit 1
  int conv_iter;     // iterations run when the pattern froze (-1: never)
  double stop;       // this pattern's stop R-factor (0: the run's stop_rfactor)
  double rmin;       // lowest in-loop R-factor of the run (reset to +inf by run_begin)
  double rbest;      // plateau stop: the R-factor of the last improvement by the tolerance
  int best_iter;     // plateau stop: iteration of that improvement
};

// Per-pattern PRTF state (phaseRetrieve's phi0 and the phase of the current step).
struct PrtfState {
  float phi0;        // -arg(sum gamma0^2)/2 at prtfIter
  float theta;       // phase added to this step's P_M Psi
};

struct RowArgs {
  const float2* in;        // rows to load
  float2* out;             // rows to store (may alias in when the layouts match)
  float2* rho;             // ROW_ITER: real-space iterate (row-major), updated in place
  const uint32_t* mask;    // ROW_ITER: support bits, (cols+31)/32 words per row
  const float2* tw;        // per-pass twiddles of length cols
  int rows;                // lines per pattern
  int mode;                // ROW_FFT / ROW_ITER
  int inv;                 // ROW_FFT direction
  int algo;                // ROW_ITER update
  int in_tiled, out_tiled; // 0: row-major, 1: column-tiled with width 1 << tile_log2
  int tile_log2;
  long long in_stride;     // elements between patterns
  long long out_stride;
  long long rho_stride;
  long long mask_stride;   // mask words between patterns
  const PatState* state;   // optional: CTAs of frozen patterns (flags bit 2) return at once
  int tc;                  // 1: radix-16 passes on the tensor cores (BF16 split, FP32 accumulate)
  float scale;             // factor applied on store (1 = none)
  float inv_n;             // 1/(rows*cols) (applyNorm after the inverse FFT)
  float beta;              // vars.beta_HIO
  int cb_plus1;            // 0: default butterfly chunk bits; k + 1: chunk bits k (autotuner)
  int pdl_mode;            // 0: the per-length default, 1: plain launch, 2: programmatic dependent launch
  int* err;                // optional: bit 0 set when a bulk copy's wait ran out
};

struct ColArgs {
  const float2* in;        // columns to load
  float2* out;             // columns to store (may alias in when the layouts match)
  float2* psi_out;         // COL_ITER: optional row-major copy of P_M(Psi), the projected Psi
  const float* amp;        // sqrt(max(I,0)), column-tiled (width = the kernel's L)
  const float* inten;      // I, column-tiled (PROJ_CCD)
  const float* bs;         // beamstop, column-tiled (PROJ_CCD), may be null
  double* rf_partials;     // optional: per-CTA sum | |Psi| - sqrt(I) |
  const float2* tw;        // per-pass twiddles of length rows
  int cols;                // lines per pattern
  int mode;                // COL_FFT / COL_ITER
  int inv;                 // COL_FFT direction
  int from_psi;            // COL_ITER: input already holds Psi (skip the forward FFT)
  int proj;                // PROJ_MODABS / PROJ_CCD
  int noise_level;
  int in_tiled, out_tiled; // 0: row-major, 1: column-tiled with width L
  long long in_stride, out_stride, aux_stride, psi_stride;
  PatState* state;         // optional: patterns with flags bit 1 freeze (bit 2), frozen ones return at once
  int tc;                  // 1: radix-16 passes on the tensor cores (BF16 split, FP32 accumulate)
  float scale;
  float ccd_scale;         // vars.scale
  float ccd_rcolor;        // vars.rcolor
  int pdl_mode;            // as RowArgs::pdl_mode
  int* err;                // as RowArgs::err
};

// Launch helpers exported by the per-size translation units.
typedef cudaError_t (*PrepLaunch)();
typedef cudaError_t (*RowLaunch)(const RowArgs&, int batch, cudaStream_t);
typedef cudaError_t (*ColLaunch)(const ColArgs&, int batch, cudaStream_t);

PrepLaunch prep_launcher(int n);   // nullptr: unsupported length
RowLaunch row_launcher(int n);
ColLaunch col_launcher(int n);
int lines_per_cta(int n);          // lines (rows or columns) per CTA for length n
int twiddle_count(int n);          // entries of the per-pass twiddle table of length n
int row_cb_default(int n, int tile_log2);   // butterfly chunk bits the row pass uses on tiled data
int row_cb_max(int n);                      // largest valid chunk bits of length n
// host: fill the per-pass twiddle table of length n (double precision, rounded once)
void twiddle_table(int n, float2* out);
// host: multiprocessors of the current device (queried once per device)
int sm_count();

}  // namespace cdx
