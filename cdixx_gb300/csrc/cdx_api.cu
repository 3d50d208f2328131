// C ABI of the CDI phase-retrieval path (include/cdx.h).
//
// A context owns one device arena per (size, batch): the real-space iterate
// rho, the work buffer W (X = rowFFT(rho) between iterations), Psi, the
// pattern I and sqrt(I), the float support field, the support bits, twiddle
// tables, reduction partials and per-pattern state.  cdx_run turns the
// algorithm string into a step list and enqueues it on the context's stream,
// captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <tuple>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cdx.h"
#include "cdx_fft.cuh"
#include "cdx_host.h"
#include "cdx_misc.h"
#include "cdx_types.h"

using namespace cdx;

#define CDX_CK(call)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return set_error(CDX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

namespace {

// Fixed partial counts of the reductions (one per SM and four per SM of a GB300):
// fixed rather than queried so that the summation order, and with it every
// reduced value, is the same on any device.
constexpr int kRedBlocks = 152;   // reduction CTAs per pattern
constexpr int kSwBlocks = 608;    // shrinkwrap y-pass CTAs per pattern

// ---------------------------------------------------------------- twiddles
// Per-pass twiddle table of length n (cdx_dispatch.cu), one per (device, n),
// kept for the life of the process.
std::mutex g_tw_mu;
std::map<std::pair<int, int>, float2*> g_tw;

int twiddles(int n, float2** out) {
  int dev = 0;
  CDX_CK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_tw_mu);
  auto it = g_tw.find({dev, n});
  if (it != g_tw.end()) { *out = it->second; return CDX_OK; }
  const int cnt = std::max(1, twiddle_count(n));
  std::vector<float2> h(cnt, make_float2(1.f, 0.f));
  twiddle_table(n, h.data());
  float2* d = nullptr;
  CDX_CK(cudaMalloc(&d, sizeof(float2) * cnt));
  CDX_CK(cudaMemcpy(d, h.data(), sizeof(float2) * cnt, cudaMemcpyHostToDevice));
  g_tw[{dev, n}] = d;
  *out = d;
  return CDX_OK;
}

}  // namespace

namespace cdx {
int device_twiddles(int n, float2** out) { return twiddles(n, out); }
}  // namespace cdx

namespace {

int check_len(int n) {
  if (!size_supported(n) || n > 4096 || !prep_launcher(n))
    return set_error(CDX_ERR_SIZE, "unsupported length " + std::to_string(n) +
                                       " (supported: 2^a 3^b in [16, 4096])");
  return CDX_OK;
}

}  // namespace

struct cdx_ctx {
  cdx_params p{};
  int rows = 0, cols = 0, batch = 0;
  long long npx = 0;
  int wpr = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  int device = 0;

  // rho, psi, tmp, inten, spt, bs: row-major (npx per pattern);
  // work, amp_t, inten_t, bs_t: column-tiled, tile width 2^tl (wstride per pattern)
  float2 *rho = nullptr, *work = nullptr, *psi = nullptr, *tmp = nullptr;
  float *inten = nullptr, *amp_t = nullptr, *inten_t = nullptr, *spt = nullptr, *bs = nullptr, *bs_t = nullptr;
  int tl = 0;              // log2 of the column-pass lines per CTA
  int cp = 0;              // cols padded to a multiple of 2^tl
  long long wstride = 0;   // rows * cp
  uint32_t* mask = nullptr;
  float2 *tw_r = nullptr, *tw_c = nullptr;   // lengths rows (column pass) and cols (row pass)
  double* part = nullptr;                    // [batch][part_per_pat]
  float* pmax = nullptr;                     // [batch][kSwBlocks]
  int part_per_pat = 0;
  int col_blocks = 0;
  PatState* dstate = nullptr;
  float* weights = nullptr;
  size_t weights_cap = 0;
  void* arena = nullptr;
  size_t arena_bytes = 0;

  // host state
  std::vector<char> have_pattern;
  std::vector<char> fresh;    // initial iterate set since the last run
  bool have_initial = false;
  bool psi_in_work = false;   // psi holds Psi0 and W nothing yet: the next iteration starts from psi
  int sx = 0, sy = 0, ex = 0, ey = 0;

  // PRTF (prtf_iter >= 0): projected Psi, rho' = IFFT(P_M Psi)/N, the ER cache,
  // gamma0, the phasor sum, the prtfIter mask; polar sums [batch][2][rows/2]
  float2 *pr_psi = nullptr, *pr_rhop = nullptr, *pr_cache = nullptr, *pr_gamma0 = nullptr, *pr_map = nullptr;
  float* pr_mask = nullptr;
  float* pr_polar = nullptr;
  double* pr_part = nullptr;
  PrtfState* pr_state = nullptr;
  bool pr_valid = false;       // the last run reached prtf_iter
  bool pr_reached = false;     // set while enqueueing

  // launch variant (autotune): RowArgs/ColArgs knobs, and what was measured
  int tune_pdl_col = 0, tune_pdl_row = 0, tune_cb_plus1 = 0;   // pdl: 0 per-length default, 1 plain, 2 PDL
  int* derr = nullptr;        // bulk-copy wait timeouts of the pass kernels (bit 0)
  bool tuned = false;
  std::string tune_report;

  // graph cache
  std::string gkey;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int last_steps = 0, last_iters = 0, last_sw = 0, last_launches = 0;
};

namespace {

void rect_of(cdx_ctx* c) {
  // createSupport (src/post_gpu/cdi.cc:240-245): double arithmetic, truncated to int
  const double o = c->p.oversampling_spt;
  c->sx = (int)((o - 1) / 2 * c->rows / o - 1);
  c->sy = (int)((o - 1) / 2 * c->cols / o - 1);
  c->ex = c->rows - c->sx;
  c->ey = c->cols - c->sy;
}

int reset_support(cdx_ctx* c, int idx, int count) {
  const long long off = (long long)idx * c->npx;
  CDX_CK(rect_support(c->spt + off, c->rows, c->cols, count, c->sx, c->sy, c->ex, c->ey, c->st));
  // bits with the current threshold of each pattern
  CDX_CK(support_bits(c->spt + off, c->dstate + idx, 0.f, c->mask + (long long)idx * c->rows * c->wpr, c->rows,
                      c->cols, count, c->st));
  return CDX_OK;
}

int copy_in(void* dst, const void* src, size_t bytes, int where, cudaStream_t st) {
  CDX_CK(cudaMemcpyAsync(dst, src, bytes, where == CDX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  return CDX_OK;
}
int copy_out(void* dst, const void* src, size_t bytes, int where, cudaStream_t st) {
  CDX_CK(cudaMemcpyAsync(dst, src, bytes, where == CDX_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
  CDX_CK(cudaStreamSynchronize(st));
  return CDX_OK;
}

// Shrinkwrap width schedule and the 1-D kernels of every shrinkwrap of a run.
struct SwPlan {
  std::vector<float> w;       // concatenated weights
  std::vector<int> offx, radx, offy, rady;
};

// Periodic kernel equal to the inverse DFT of the sampled frequency Gaussian
// exp(-f^2/(2 sf^2)) (f in FFT order) that applyGaussMult multiplies Psi by
// (src/gpu/cudaConfig.cu:380-395); truncated at the smallest radius whose
// dropped tail holds at most 2e-8 of the kernel's absolute mass (below float32
// resolution of the blurred field), at most 64.  The Gaussian is cut at the
// Nyquist frequency, so the kernel rings: a pointwise 1e-10 cut would need
// r = 50 at sigma = 3 where this one needs 12.
void fourier_kernel(int n, double sf, std::vector<float>& w, int& off, int& rad) {
  // the sigma schedule repeats every run: cache the truncated kernel per (n, sf)
  static std::mutex mu;
  static std::map<std::pair<int, double>, std::vector<float>> cache;
  std::vector<float> taps;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find({n, sf});
    if (it != cache.end()) taps = it->second;
  }
  if (taps.empty()) {
    const int half = n / 2;
    std::vector<double> k(half + 1), ct(n), g(n);
    const double two_pi = 6.283185307179586476925286766559;
    for (int t = 0; t < n; ++t) ct[t] = std::cos(two_pi * (double)t / n);
    for (int f = 0; f < n; ++f) {
      const int fr = f >= n / 2 ? f - n : f;
      g[f] = std::exp(-(double)fr * fr / (2.0 * sf * sf));
    }
    for (int m = 0; m <= half; ++m) {
      double s = 0.0;
      for (int f = 0; f < n; ++f) s += g[f] * ct[(int)(((long long)f * m) % n)];
      k[m] = s / n;
    }
    // absolute mass of the whole periodic kernel (k is even: k[m] = k[n - m])
    double total = 0.0;
    for (int m = 0; m < n; ++m) total += std::fabs(k[m <= half ? m : n - m]);
    const int rmax = std::min((n - 1) / 2, 64);
    double kept = std::fabs(k[0]);
    int r = 0;
    while (r < rmax && total - kept > 2e-8 * total) {
      ++r;
      kept += 2.0 * std::fabs(k[r]);
    }
    for (int d = -r; d <= r; ++d) taps.push_back((float)k[d < 0 ? -d : d]);
    std::lock_guard<std::mutex> lk(mu);
    cache[{n, sf}] = taps;
  }
  off = (int)w.size();
  rad = ((int)taps.size() - 1) / 2;
  w.insert(w.end(), taps.begin(), taps.end());
}

// Normalised sampled Gaussian of width sigma px, radius floor(6 sigma)/2 as
// applyGaussConv sizes it (src/post_gpu/misc.cc:80-86).
void spatial_kernel(int n, double sigma, std::vector<float>& w, int& off, int& rad) {
  int r = ((int)std::floor(sigma * 6)) >> 1;
  r = std::max(0, std::min(std::min(r, (n - 1) / 2), 64));   // 64: the stencil kernels' largest radius
  std::vector<double> k(2 * r + 1);
  double s = 0.0;
  for (int d = -r; d <= r; ++d) s += (k[d + r] = std::exp(-(double)d * d / (2.0 * sigma * sigma)));
  off = (int)w.size();
  rad = r;
  for (int d = -r; d <= r; ++d) w.push_back((float)(k[d + r] / s));
}

void plan_shrinkwrap(const cdx_ctx* c, int count, SwPlan& P) {
  float g = c->p.sigma0;
  for (int i = 0; i < count; ++i) {
    int ox, rx, oy, ry;
    if (c->p.shrink_mode == CDX_SHRINK_FOURIER) {
      // sigma_f = Real(row>>2)/gaussianSigma in float (cdi.cc:327), same for both axes
      const float sf = (float)(c->rows >> 2) / g;
      fourier_kernel(c->rows, sf, P.w, ox, rx);
      fourier_kernel(c->cols, sf, P.w, oy, ry);
    } else {
      spatial_kernel(c->rows, g, P.w, ox, rx);
      spatial_kernel(c->cols, g, P.w, oy, ry);
    }
    P.offx.push_back(ox); P.radx.push_back(rx); P.offy.push_back(oy); P.rady.push_back(ry);
    if (g > c->p.sigma_min) g = (float)((double)g * (double)c->p.sigma_decay);   // gaussianSigma*=0.99
  }
}

int col_iter(cdx_ctx* c, bool from_psi, bool rf, float2* psi_proj = nullptr) {
  ColArgs a{};
  // the first iteration after a restart reads Psi0 (row-major) from psi
  a.in = from_psi ? c->psi : c->work;
  a.in_tiled = from_psi ? 0 : 1;
  a.in_stride = from_psi ? c->npx : c->wstride;
  a.out = c->work;
  a.out_tiled = 1;
  a.out_stride = c->wstride;
  a.psi_out = psi_proj;
  a.psi_stride = c->npx;
  a.amp = c->amp_t;
  a.inten = c->inten_t;
  a.bs = c->bs_t;
  a.aux_stride = c->wstride;
  a.state = c->dstate;
  a.tc = c->p.fft_mode;
  a.rf_partials = rf ? c->part : nullptr;
  a.tw = c->tw_r;
  a.cols = c->cols;
  a.mode = COL_ITER;
  a.from_psi = from_psi;
  a.proj = c->p.sim_ccd_bit ? PROJ_CCD : PROJ_MODABS;
  a.noise_level = c->p.noise_level;
  a.scale = 1.f;
  a.ccd_scale = 1.f / c->p.exposure;
  a.ccd_rcolor = (float)c->p.rcolor;
  a.pdl_mode = c->tune_pdl_col;
  a.err = c->derr;
  CDX_CK(col_launcher(c->rows)(a, c->batch, c->st));
  return CDX_OK;
}

int row_iter(cdx_ctx* c, int algo) {
  RowArgs a{};
  a.in = c->work;
  a.out = c->work;
  a.in_tiled = a.out_tiled = 1;
  a.tile_log2 = c->tl;
  a.in_stride = a.out_stride = c->wstride;
  a.rho = c->rho;
  a.rho_stride = c->npx;
  a.mask = c->mask;
  a.mask_stride = (long long)c->rows * c->wpr;
  a.state = c->dstate;
  a.tc = c->p.fft_mode;
  a.tw = c->tw_c;
  a.rows = c->rows;
  a.mode = ROW_ITER;
  a.algo = algo;
  a.scale = 1.f;
  a.inv_n = (float)(1.0 / ((double)c->rows * c->cols));   // applyNorm(.., 1./(row*column)), cdi.cc:353
  a.beta = c->p.beta;
  a.cb_plus1 = c->tune_cb_plus1;
  a.pdl_mode = c->tune_pdl_row;
  a.err = c->derr;
  CDX_CK(row_launcher(c->cols)(a, c->batch, c->st));
  return CDX_OK;
}

// Generic 2-D transform of `batch` row-major patterns: rows then columns.
int fft2_enqueue(const float2* in, float2* out, int rows, int cols, int batch, bool inv, float scale,
                 const float2* tw_rows_len, const float2* tw_cols_len, cudaStream_t st, int tc = 0) {
  const long long n = (long long)rows * cols;
  RowArgs r{};
  r.in = in;
  r.out = out;
  r.in_stride = r.out_stride = n;
  r.tw = tw_cols_len;
  r.rows = rows;
  r.mode = ROW_FFT;
  r.inv = inv;
  r.tc = tc;
  r.scale = 1.f;
  CDX_CK(row_launcher(cols)(r, batch, st));
  ColArgs c{};
  c.in = out;
  c.out = out;
  c.in_stride = c.out_stride = n;
  c.tw = tw_rows_len;
  c.cols = cols;
  c.mode = COL_FFT;
  c.inv = inv;
  c.tc = tc;
  c.scale = scale;
  CDX_CK(col_launcher(rows)(c, batch, st));
  return CDX_OK;
}

// Enqueue one whole phaseRetrieve on c->st (no synchronisation).
int enqueue_run(cdx_ctx* c, const std::vector<int>& steps, const SwPlan& sw, bool psi_in_work) {
  const long long n_all = c->npx * c->batch;
  const float sqn = (float)std::sqrt((double)c->rows * c->cols);
  int nl = 0;   // kernels enqueued
  CDX_CK(run_begin(c->dstate, c->batch, c->st));
  ++nl;
  // applyNorm(cuda_gkp1, 1./sqrt(row*column)) at the start (cdi.cc:313)
  CDX_CK(scale_complex(c->rho, (float)(1.0 / std::sqrt((double)c->rows * c->cols)), n_all, c->st));
  ++nl;
  bool from_psi = psi_in_work;
  int it = 0, swi = 0, step = -1;
  const bool prtf = c->pr_map && c->p.prtf_iter >= 0;
  c->pr_reached = false;
  if (prtf) CDX_CK(cudaMemsetAsync(c->pr_map, 0, sizeof(float2) * n_all, c->st));
  for (int a : steps) {
    ++step;   // phaseRetrieve's iter: every step, shrinkwraps included
    if (a == ALGO_SHRINKWRAP) {
      const bool m2 = c->p.shrink_mode == CDX_SHRINK_SPATIAL;
      CDX_CK(shrinkwrap(c->rho, c->tmp, c->spt, c->weights + sw.offx[swi], sw.radx[swi], c->weights + sw.offy[swi],
                        sw.rady[swi], c->rows, c->cols, c->batch, m2, (float)((double)c->rows * c->cols), c->pmax,
                        c->part, kSwBlocks, c->dstate, c->p.shrink_threshold, c->st));
      CDX_CK(support_bits(c->spt, c->dstate, 0.f, c->mask, c->rows, c->cols, c->batch, c->st));
      nl += 4;
      ++swi;
      continue;
    }
    // from iteration 1 on: the restart iterate has the measured modulus by construction
    const bool rf = c->p.rf_every > 0 && it > 0 && (it % c->p.rf_every) == 0;
    const bool pstep = prtf && step >= c->p.prtf_iter;
    int e = col_iter(c, from_psi, rf, pstep ? c->pr_psi : nullptr);
    if (e) return e;
    if (rf)
      CDX_CK(rfactor_from_partials(c->part, c->col_blocks, c->batch, c->dstate, c->p.stop_rfactor, it,
                                   c->p.plateau_iters, c->p.plateau_tol, c->st));
    e = row_iter(c, a);
    if (e) return e;
    nl += rf ? 3 : 2;
    if (pstep) {
      // cdi.cc:355-380: rho' = IFFT(P_M Psi)/N, the ER correlation with gamma0, its
      // phase, and the phasor accumulation of P_M Psi
      const bool first = step == c->p.prtf_iter;
      e = fft2_enqueue(c->pr_psi, c->pr_rhop, c->rows, c->cols, c->batch, true,
                       (float)(1.0 / ((double)c->rows * c->cols)), c->tw_r, c->tw_c, c->st);
      if (e) return e;
      CDX_CK(prtf_step(c->pr_rhop, c->mask, c->rows, c->cols, c->batch, c->pr_cache, c->pr_gamma0, first, c->pr_part,
                       kRedBlocks, c->pr_state, c->dstate, c->st));
      CDX_CK(prtf_accum(c->pr_psi, c->pr_map, first ? c->pr_mask : nullptr, c->npx, c->batch, c->pr_state, c->dstate,
                        c->st));
      if (first) {
        CDX_CK(prtf_polar(c->pr_mask, nullptr, 1.f, c->rows, c->cols, c->batch, c->pr_polar, c->st));
        c->pr_reached = true;
      }
      nl += first ? 6 : 5;
    }
    from_psi = false;
    ++it;
  }
  if (prtf && c->pr_reached) {
    // |prtf_map| / (iter - prtfIter), polar sums (cdi.cc:424-433)
    const float inv = (float)(1.0 / ((double)(step + 1) - c->p.prtf_iter));
    CDX_CK(prtf_polar(nullptr, c->pr_map, inv, c->rows, c->cols, c->batch, c->pr_polar + c->batch * (c->rows / 2),
                      c->st));
    ++nl;
  }
  // final Psi = FFT(rho): W holds rowFFT(rho); with no iteration psi still holds Psi0
  if (!(it == 0 && psi_in_work)) {
    ColArgs a{};
    a.in = c->work;
    a.in_tiled = 1;
    a.in_stride = c->wstride;
    a.out = c->psi;
    a.out_tiled = 0;
    a.out_stride = c->npx;
    a.tw = c->tw_r;
    a.cols = c->cols;
    a.mode = COL_FFT;
    a.inv = 0;
    a.tc = c->p.fft_mode;
    a.scale = 1.f;
    CDX_CK(col_launcher(c->rows)(a, c->batch, c->st));
    ++nl;
  }
  // applyNorm(cuda_gkp1, sqrt(row*column)) (cdi.cc:406)
  CDX_CK(scale_complex(c->rho, sqn, n_all, c->st));
  CDX_CK(residual_rfactor(c->psi, c->inten, c->npx, c->batch, c->part, kRedBlocks, c->dstate, c->st));
  nl += 3;
  c->last_launches = nl;
  return CDX_OK;
}

int prepare_run(cdx_ctx* c, const char* algorithm, std::vector<int>& steps, SwPlan& sw) {
  if (!c) return set_error(CDX_ERR_ARG, "null context");
  for (int i = 0; i < c->batch; ++i)
    if (!c->have_pattern[i]) return set_error(CDX_ERR_STATE, "pattern " + std::to_string(i) + " not set");
  if (!c->have_initial) return set_error(CDX_ERR_STATE, "no initial iterate (cdx_set_initial / cdx_random_start)");
  int nfresh = 0;
  for (char f : c->fresh) nfresh += f;
  if (nfresh != 0 && nfresh != c->batch)
    return set_error(CDX_ERR_STATE, "a batch restarts together: set the initial iterate of every pattern");
  int e = algo_expand(algorithm, steps, 50000000);
  if (e) return e;
  int nsw = 0;
  for (int a : steps) {
    if (a == ALGO_TV) return set_error(CDX_ERR_ALGO, "TV step (FISTA denoising) is not part of this path");
    nsw += a == ALGO_SHRINKWRAP;
  }
  plan_shrinkwrap(c, nsw, sw);
  if (!sw.w.empty()) {
    if (sw.w.size() > c->weights_cap) {
      if (c->weights) cudaFree(c->weights);
      c->weights = nullptr;
      c->weights_cap = 0;
      CDX_CK(cudaMalloc(&c->weights, sizeof(float) * sw.w.size()));
      c->weights_cap = sw.w.size();
    }
    CDX_CK(cudaMemcpyAsync(c->weights, sw.w.data(), sizeof(float) * sw.w.size(), cudaMemcpyHostToDevice, c->st));
    CDX_CK(cudaStreamSynchronize(c->st));
  }
  c->last_steps = (int)steps.size();
  c->last_sw = nsw;
  c->last_iters = (int)steps.size() - nsw;
  return CDX_OK;
}

// Autotuner: before the first run of a context with autotune set, time the
// iteration (column pass + row pass, HIO; eight of them captured in a graph,
// as runs execute) under each launch variant -- programmatic dependent launch
// off/on for the column pass and for the row pass, x the row pass's butterfly
// chunk bits (the default and up to two below it) -- on a copy of the
// context's own state, restore the state, and keep the fastest.  Decisions are
// cached per (device, rows, cols, batch) for the process, and can be saved to
// and loaded from a JSON file (cdx_tuning_save / cdx_tuning_load), where they
// are keyed by the device's name so that they carry over to the same model.
struct TuneRec {
  int pdl_col = 0, pdl_row = 0, cb_plus1 = 0;
  double us = 0.0;
};
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, TuneRec> g_tune;                   // (device, rows, cols, batch)
std::map<std::tuple<std::string, int, int, int>, TuneRec> g_tune_named;    // (device name, rows, cols, batch)

std::string device_name(int dev) {
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
    cudaGetLastError();
    return std::string();
  }
  return std::string(prop.name);
}

int autotune(cdx_ctx* c) {
  const auto key = std::make_tuple(c->device, c->rows, c->cols, c->batch);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    const char* how = "cached";
    if (it == g_tune.end()) {
      auto nt = g_tune_named.find(std::make_tuple(device_name(c->device), c->rows, c->cols, c->batch));
      if (nt != g_tune_named.end()) {
        it = g_tune.emplace(key, nt->second).first;
        how = "loaded";
      }
    }
    if (it != g_tune.end()) {
      c->tune_pdl_col = it->second.pdl_col;
      c->tune_pdl_row = it->second.pdl_row;
      c->tune_cb_plus1 = it->second.cb_plus1;
      c->tuned = true;
      c->tune_report = how;
      return CDX_OK;
    }
  }
  if (c->p.fft_mode != CDX_FFT_FP32) {   // the tensor-core kernels have neither knob
    c->tuned = true;
    return CDX_OK;
  }
  const size_t nrho = (size_t)c->npx * c->batch, nw = (size_t)c->wstride * c->batch;
  // copies of the state the timed iterations overwrite, freed on every path
  struct Scratch {
    float2 *rho = nullptr, *w = nullptr;
    ~Scratch() {
      if (rho) cudaFree(rho);
      if (w) cudaFree(w);
    }
  } save;
  if (cudaMalloc(&save.rho, sizeof(float2) * nrho) != cudaSuccess || cudaMalloc(&save.w, sizeof(float2) * nw) != cudaSuccess) {
    cudaGetLastError();
    return set_error(CDX_ERR_NOMEM, "autotune: no room for a copy of the state");
  }
  float2* const srho = save.rho;
  float2* const sw = save.w;
  CDX_CK(cudaMemcpyAsync(srho, c->rho, sizeof(float2) * nrho, cudaMemcpyDeviceToDevice, c->st));
  CDX_CK(cudaMemcpyAsync(sw, c->work, sizeof(float2) * nw, cudaMemcpyDeviceToDevice, c->st));
  const int cbd = row_cb_default(c->cols, c->tl);
  TuneRec best;
  best.us = 1e30;
  std::string rep;
  int e = CDX_OK;
  for (int pc = 1; pc <= 2 && e == CDX_OK; ++pc)
    for (int pr = 1; pr <= 2 && e == CDX_OK; ++pr)
      for (int cb = cbd; cb >= std::max(0, cbd - 2) && e == CDX_OK; --cb) {
        c->tune_pdl_col = pc;
        c->tune_pdl_row = pr;
        c->tune_cb_plus1 = cb + 1;
        // timed as the runs execute: kTimed iterations captured in one graph,
        // launched once to warm up and once under the events
        constexpr int kTimed = 8;
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        CDX_CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
        for (int i = 0; i < kTimed && e == CDX_OK; ++i) {
          e = col_iter(c, false, false);
          if (e == CDX_OK) e = row_iter(c, ALGO_HIO);
        }
        const cudaError_t ce = cudaStreamEndCapture(c->st, &g);
        if (e == CDX_OK && ce != cudaSuccess) e = set_error(CDX_ERR_CUDA, std::string("autotune capture: ") + cudaGetErrorString(ce));
        if (e == CDX_OK && cudaGraphInstantiate(&ge, g, 0) != cudaSuccess) e = set_error(CDX_ERR_CUDA, "autotune graph");
        if (g) cudaGraphDestroy(g);
        float ms = 0.f;
        if (e == CDX_OK) {
          cudaError_t le = cudaGraphLaunch(ge, c->st);
          if (le == cudaSuccess) le = cudaEventRecord(c->ev0, c->st);
          if (le == cudaSuccess) le = cudaGraphLaunch(ge, c->st);
          if (le == cudaSuccess) le = cudaEventRecord(c->ev1, c->st);
          if (le == cudaSuccess) le = cudaEventSynchronize(c->ev1);
          if (le == cudaSuccess) le = cudaEventElapsedTime(&ms, c->ev0, c->ev1);
          if (le != cudaSuccess) e = set_error(CDX_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(le));
        }
        if (ge) cudaGraphExecDestroy(ge);
        if (e != CDX_OK) break;
        const double us = 1000.0 * ms / kTimed;
        char line[128];
        snprintf(line, sizeof line, "pdl_col=%d pdl_row=%d chunk=%d: %.2f us\n", pc - 1, pr - 1, cb, us);
        rep += line;
        if (us < best.us) {
          best.us = us;
          best.pdl_col = pc;
          best.pdl_row = pr;
          best.cb_plus1 = cb + 1;
        }
      }
  // restore the state the runs iterated on
  if (e == CDX_OK) {
    CDX_CK(cudaMemcpyAsync(c->rho, srho, sizeof(float2) * nrho, cudaMemcpyDeviceToDevice, c->st));
    CDX_CK(cudaMemcpyAsync(c->work, sw, sizeof(float2) * nw, cudaMemcpyDeviceToDevice, c->st));
    CDX_CK(cudaStreamSynchronize(c->st));
  }
  if (e != CDX_OK) return e;
  c->tune_pdl_col = best.pdl_col;
  c->tune_pdl_row = best.pdl_row;
  c->tune_cb_plus1 = best.cb_plus1;
  c->tuned = true;
  c->tune_report = rep;
  const std::string name = device_name(c->device);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = best;
  if (!name.empty()) g_tune_named[std::make_tuple(name, c->rows, c->cols, c->batch)] = best;
  return CDX_OK;
}

// ---------------------------------------------------------- tuning file (JSON)
// {"cdx_tuning": 1, "entries": [{"device": "<name>", "rows": R, "cols": C,
//   "batch": B, "pdl_col": 0|1, "pdl_row": 0|1, "row_chunk_bits": k, "us": t}, ...]}
// A small reader for exactly this shape: flat objects of string and number
// values inside the "entries" array; anything else is an error.
struct JsonLex {
  const std::string& t;
  size_t i = 0;
  explicit JsonLex(const std::string& s) : t(s) {}
  void ws() {
    while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t')) ++i;
  }
  bool eat(char ch) {
    ws();
    if (i < t.size() && t[i] == ch) {
      ++i;
      return true;
    }
    return false;
  }
  bool str(std::string& out) {
    ws();
    if (i >= t.size() || t[i] != '"') return false;
    out.clear();
    for (++i; i < t.size() && t[i] != '"'; ++i) {
      if (t[i] == '\\' && i + 1 < t.size()) ++i;
      out.push_back(t[i]);
    }
    if (i >= t.size()) return false;
    ++i;
    return true;
  }
  bool num(double& v) {
    ws();
    const char* b = t.c_str() + i;
    char* e = nullptr;
    v = std::strtod(b, &e);
    if (e == b) return false;
    i += (size_t)(e - b);
    return true;
  }
};

int parse_tuning(const std::string& text, std::vector<std::pair<std::string, std::pair<std::tuple<int, int, int>, TuneRec>>>& out) {
  JsonLex L(text);
  std::string k;
  double v = 0;
  if (!L.eat('{')) return set_error(CDX_ERR_IO, "tuning file: expected '{'");
  bool entries = false;
  do {
    if (!L.str(k) || !L.eat(':')) return set_error(CDX_ERR_IO, "tuning file: expected a key");
    if (k == "entries") {
      if (!L.eat('[')) return set_error(CDX_ERR_IO, "tuning file: entries must be an array");
      entries = true;
      if (L.eat(']')) continue;
      do {
        if (!L.eat('{')) return set_error(CDX_ERR_IO, "tuning file: expected an entry object");
        std::string dev;
        int rows = 0, cols = 0, batch = 0, pc = -1, pr = -1, cb = -1;
        double us = 0;
        do {
          if (!L.str(k) || !L.eat(':')) return set_error(CDX_ERR_IO, "tuning file: expected an entry key");
          if (k == "device") {
            if (!L.str(dev)) return set_error(CDX_ERR_IO, "tuning file: device must be a string");
          } else {
            if (!L.num(v)) return set_error(CDX_ERR_IO, "tuning file: expected a number for " + k);
            if (k == "rows") rows = (int)v;
            else if (k == "cols") cols = (int)v;
            else if (k == "batch") batch = (int)v;
            else if (k == "pdl_col") pc = (int)v;
            else if (k == "pdl_row") pr = (int)v;
            else if (k == "row_chunk_bits") cb = (int)v;
            else if (k == "us") us = v;
          }
        } while (L.eat(','));
        if (!L.eat('}')) return set_error(CDX_ERR_IO, "tuning file: expected '}'");
        if (dev.empty() || !cdx_size_supported(rows) || !cdx_size_supported(cols) || batch < 1 || pc < 0 ||
            pc > 1 || pr < 0 || pr > 1 || cb < 0 || cb > row_cb_max(cols))
          return set_error(CDX_ERR_IO, "tuning file: entry out of range");
        TuneRec r;
        r.pdl_col = pc + 1;
        r.pdl_row = pr + 1;
        r.cb_plus1 = cb + 1;
        r.us = us;
        out.push_back({dev, {std::make_tuple(rows, cols, batch), r}});
      } while (L.eat(','));
      if (!L.eat(']')) return set_error(CDX_ERR_IO, "tuning file: expected ']'");
    } else if (!L.num(v)) {
      std::string skip;
      if (!L.str(skip)) return set_error(CDX_ERR_IO, "tuning file: unexpected value for " + k);
    }
  } while (L.eat(','));
  if (!L.eat('}') || !entries) return set_error(CDX_ERR_IO, "tuning file: expected an \"entries\" array");
  return CDX_OK;
}

int run_impl(cdx_ctx* c, const char* algorithm) {
  std::vector<int> steps;
  SwPlan sw;
  int e = prepare_run(c, algorithm, steps, sw);
  if (e) return e;
  CDX_CK(cudaSetDevice(c->device));
  if (c->p.autotune && !c->tuned && c->last_iters > 0 && (e = autotune(c))) return e;
  const bool piw = c->psi_in_work;
  if (c->p.use_graph) {
    char key[64];
    snprintf(key, sizeof key, "|%d|%p", (int)piw, (void*)c->weights);
    std::string k = std::string(algorithm) + key;
    if (k != c->gkey || !c->gexec) {
      if (c->gexec) { cudaGraphExecDestroy(c->gexec); c->gexec = nullptr; }
      c->gkey.clear();
      cudaGraph_t g = nullptr;
      CDX_CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      e = enqueue_run(c, steps, sw, piw);
      cudaError_t ce = cudaStreamEndCapture(c->st, &g);
      if (e) { if (g) cudaGraphDestroy(g); return e; }
      if (ce != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
      ce = cudaGraphInstantiate(&c->gexec, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
      c->gkey = k;
    }
    CDX_CK(cudaEventRecord(c->ev0, c->st));
    CDX_CK(cudaGraphLaunch(c->gexec, c->st));
    CDX_CK(cudaEventRecord(c->ev1, c->st));
  } else {
    CDX_CK(cudaEventRecord(c->ev0, c->st));
    e = enqueue_run(c, steps, sw, piw);
    if (e) return e;
    CDX_CK(cudaEventRecord(c->ev1, c->st));
  }
  if (c->last_iters > 0) c->psi_in_work = false;
  c->pr_valid = c->pr_reached;
  c->fresh.assign(c->batch, 0);
  return CDX_OK;
}

}  // namespace

// A set of contexts run as one CUDA graph, one branch per context: the branches
// one after another (default) or side by side (concurrent).
struct cdx_group {
  std::vector<cdx_ctx*> ctxs;
  int concurrent = 0;
  cudaStream_t st = nullptr;
  cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t gexec = nullptr;
  std::string gkey;
};

namespace {

int group_run_impl(cdx_group* g, const char* algorithm, double* gpu_ms) {
  const size_t n = g->ctxs.size();
  std::vector<std::vector<int>> steps(n);
  std::vector<SwPlan> sw(n);
  std::string key = algorithm;
  key += g->concurrent ? "|concurrent" : "|serial";
  for (size_t i = 0; i < n; ++i) {
    cdx_ctx* c = g->ctxs[i];
    int e = prepare_run(c, algorithm, steps[i], sw[i]);
    if (e) return e;
    char k[64];
    snprintf(k, sizeof k, "|%d|%p", (int)c->psi_in_work, (void*)c->weights);
    key += k;
  }
  if (key != g->gkey || !g->gexec) {
    if (g->gexec) { cudaGraphExecDestroy(g->gexec); g->gexec = nullptr; }
    g->gkey.clear();
    cudaGraph_t graph = nullptr;
    CDX_CK(cudaStreamBeginCapture(g->st, cudaStreamCaptureModeThreadLocal));
    int e = CDX_OK;
    cudaError_t ce = cudaEventRecord(g->fork, g->st);
    for (size_t i = 0; i < n && ce == cudaSuccess && !e; ++i) {
      cdx_ctx* c = g->ctxs[i];
      // the context's stream joins the capture: after the fork (side by side) or after the
      // previous branch (one after another)
      ce = cudaStreamWaitEvent(c->st, (g->concurrent || i == 0) ? g->fork : g->joins[i - 1], 0);
      if (ce == cudaSuccess) e = enqueue_run(c, steps[i], sw[i], c->psi_in_work);
      if (ce == cudaSuccess && !e) ce = cudaEventRecord(g->joins[i], c->st);
      if (ce == cudaSuccess && !e) ce = cudaStreamWaitEvent(g->st, g->joins[i], 0);
    }
    cudaError_t ce2 = cudaStreamEndCapture(g->st, &graph);
    if (e) { if (graph) cudaGraphDestroy(graph); return e; }
    if (ce == cudaSuccess) ce = ce2;
    if (ce != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return set_error(CDX_ERR_CUDA, std::string("group capture: ") + cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(&g->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return set_error(CDX_ERR_CUDA, std::string("group instantiate: ") + cudaGetErrorString(ce));
    g->gkey = key;
  }
  CDX_CK(cudaEventRecord(g->ev0, g->st));
  CDX_CK(cudaGraphLaunch(g->gexec, g->st));
  CDX_CK(cudaEventRecord(g->ev1, g->st));
  CDX_CK(cudaStreamSynchronize(g->st));
  for (cdx_ctx* c : g->ctxs) {
    if (c->last_iters > 0) c->psi_in_work = false;
    c->pr_valid = c->pr_reached;
    c->fresh.assign(c->batch, 0);
  }
  if (gpu_ms) {
    float ms = 0.f;
    CDX_CK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    *gpu_ms = ms;
  }
  return CDX_OK;
}

int fill_stats(cdx_ctx* c, int idx, cdx_stats* s) {
  if (!s) return CDX_OK;
  PatState h;
  CDX_CK(cudaMemcpyAsync(&h, c->dstate + idx, sizeof h, cudaMemcpyDeviceToHost, c->st));
  CDX_CK(cudaStreamSynchronize(c->st));
  memset(s, 0, sizeof *s);
  s->steps = c->last_steps;
  s->iterations = c->last_iters;
  s->shrinkwraps = c->last_sw;
  s->residual = h.residual;
  s->rfactor = h.rfactor;
  s->threshold = h.threshold;
  s->flags = h.flags;
  s->launches = c->last_launches;
  s->converged_iter = h.conv_iter;
  s->rfactor_min = h.rmin;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) s->gpu_ms = ms;
  else cudaGetLastError();
  return CDX_OK;
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

int cdx_params_default(cdx_params* p) {
  if (!p) return set_error(CDX_ERR_ARG, "null params");
  memset(p, 0, sizeof *p);
  p->batch = 1;
  p->beta = 1.f;               // vars.beta_HIO (src/gpu/cdi.cu:22)
  p->shrink_threshold = 0.f;   // readConfig default
  p->oversampling_spt = 2.f;   // html/default/cdi.cfg
  p->exposure = 1.f;
  p->rcolor = 65535;           // include/format.hpp:20
  p->shrink_mode = CDX_SHRINK_FOURIER;
  p->sigma0 = 3.f;             // cdi.cc:314
  p->sigma_min = 2.f;          // cdi.cc:338
  p->sigma_decay = 0.99f;      // cdi.cc:339
  p->use_graph = 1;
  p->rf_every = 0;
  p->plateau_iters = 0;
  p->plateau_tol = 0.01f;
  p->prtf_iter = -1;
  return CDX_OK;
}

int cdx_size_supported(int n) { return size_supported(n) && n <= 4096 ? 1 : 0; }

const char* cdx_last_error(void) { return last_error(); }
const char* cdx_version(void) { return "cdx 0.1 (sm_103a)"; }

int cdx_create(const cdx_params* p, void* stream, cdx_ctx** out) {
  if (!p || !out) return set_error(CDX_ERR_ARG, "null argument");
  *out = nullptr;
  int e = check_len(p->rows);
  if (e) return e;
  if ((e = check_len(p->cols))) return e;
  if (p->rows % 2 || p->cols % 2) return set_error(CDX_ERR_SIZE, "rows and cols must be even");
  if (p->batch < 1 || p->batch > 65535) return set_error(CDX_ERR_ARG, "batch must be in [1, 65535]");
  if (!(p->exposure > 0)) return set_error(CDX_ERR_ARG, "exposure must be > 0");
  if (!(p->oversampling_spt > 0)) return set_error(CDX_ERR_ARG, "oversampling_spt must be > 0");
  if (p->fft_mode != CDX_FFT_FP32 && p->fft_mode != CDX_FFT_TC_BF16 && p->fft_mode != CDX_FFT_TC_MMA)
    return set_error(CDX_ERR_ARG, "unknown fft_mode");
  if (p->plateau_iters < 0 || !(p->plateau_tol >= 0.f && p->plateau_tol < 1.f))
    return set_error(CDX_ERR_ARG, "plateau_iters must be >= 0 and plateau_tol in [0, 1)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(CDX_ERR_NOLIB, "no CUDA device");
  }
  cdx_ctx* c = new cdx_ctx();
  c->p = *p;
  c->rows = p->rows;
  c->cols = p->cols;
  c->batch = p->batch;
  c->npx = (long long)p->rows * p->cols;
  c->wpr = (p->cols + 31) >> 5;
  c->have_pattern.assign(p->batch, 0);
  c->fresh.assign(p->batch, 0);
  cudaGetDevice(&c->device);
  auto fail = [&](int code) { cdx_destroy(c); return code; };
  if (stream) {
    c->st = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess)
      return fail(set_error(CDX_ERR_CUDA, "stream create failed"));
    c->own_stream = true;
  }
  if (prep_launcher(c->rows)() != cudaSuccess || prep_launcher(c->cols)() != cudaSuccess || misc_prepare() != cudaSuccess)
    return fail(set_error(CDX_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString(cudaGetLastError())));
  if ((e = twiddles(c->rows, &c->tw_r)) || (e = twiddles(c->cols, &c->tw_c))) return fail(e);
  const int lc = lines_per_cta(c->rows);
  c->tl = 0;
  while ((1 << c->tl) < lc) ++c->tl;
  c->cp = (c->cols + lc - 1) / lc * lc;
  c->wstride = (long long)c->rows * c->cp;
  c->col_blocks = c->cp / lc;
  c->part_per_pat = std::max(std::max(kRedBlocks, kSwBlocks), c->col_blocks);
  // one arena: row-major rho, psi, tmp, I, support; tiled W, sqrt(I), I;
  // bits, partials, state
  const size_t B = (size_t)c->batch, N = (size_t)c->npx, W = (size_t)c->wstride;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = 0;
  const size_t o_rho = off; off += al(sizeof(float2) * B * N);
  const size_t o_work = off; off += al(sizeof(float2) * B * W);
  const size_t o_psi = off; off += al(sizeof(float2) * B * N);
  const size_t o_tmp = off; off += al(sizeof(float2) * B * N);
  const size_t o_int = off; off += al(sizeof(float) * B * N);
  const size_t o_amp = off; off += al(sizeof(float) * B * W);
  const size_t o_intt = off; off += al(sizeof(float) * B * W);
  const size_t o_spt = off; off += al(sizeof(float) * B * N);
  const size_t o_mask = off; off += al(sizeof(uint32_t) * B * c->rows * c->wpr);
  const size_t o_part = off; off += al(sizeof(double) * B * c->part_per_pat);
  const size_t o_pmax = off; off += al(sizeof(float) * B * kSwBlocks);
  const size_t o_state = off; off += al(sizeof(PatState) * B);
  const size_t o_err = off; off += al(sizeof(int));
  if (cudaMalloc(&c->arena, off) != cudaSuccess) {
    cudaGetLastError();
    return fail(set_error(CDX_ERR_NOMEM, "device arena of " + std::to_string(off) + " bytes"));
  }
  c->arena_bytes = off;
  char* a = (char*)c->arena;
  c->rho = (float2*)(a + o_rho);
  c->work = (float2*)(a + o_work);
  c->psi = (float2*)(a + o_psi);
  c->tmp = (float2*)(a + o_tmp);
  c->inten = (float*)(a + o_int);
  c->amp_t = (float*)(a + o_amp);
  c->inten_t = (float*)(a + o_intt);
  c->spt = (float*)(a + o_spt);
  c->mask = (uint32_t*)(a + o_mask);
  c->part = (double*)(a + o_part);
  c->pmax = (float*)(a + o_pmax);
  c->dstate = (PatState*)(a + o_state);
  c->derr = (int*)(a + o_err);
  if (cudaMemsetAsync(c->arena, 0, off, c->st) != cudaSuccess)
    return fail(set_error(CDX_ERR_CUDA, "arena clear failed"));
  // vars.threshold starts at 0.5 (src/gpu/cdi.cu:21)
  if (state_init(c->dstate, c->batch, 0.5f, c->st) != cudaSuccess)
    return fail(set_error(CDX_ERR_CUDA, "state init failed"));
  rect_of(c);
  if ((e = reset_support(c, 0, c->batch))) return fail(e);
  if (p->prtf_iter >= 0) {
    const size_t nb = (size_t)c->batch * c->npx;
    bool ok = cudaMalloc(&c->pr_psi, sizeof(float2) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_rhop, sizeof(float2) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_cache, sizeof(float2) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_gamma0, sizeof(float2) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_map, sizeof(float2) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_mask, sizeof(float) * nb) == cudaSuccess &&
              cudaMalloc(&c->pr_polar, sizeof(float) * 2 * c->batch * (c->rows / 2 + 1)) == cudaSuccess &&
              cudaMalloc(&c->pr_part, sizeof(double) * 2 * c->batch * kRedBlocks) == cudaSuccess &&
              cudaMalloc(&c->pr_state, sizeof(PrtfState) * c->batch) == cudaSuccess;
    if (!ok) return fail(set_error(CDX_ERR_NOMEM, "PRTF buffers"));
    // the reference's cache and gamma0 come from its pool uncleared; here they start at zero
    ok = cudaMemsetAsync(c->pr_cache, 0, sizeof(float2) * nb, c->st) == cudaSuccess &&
         cudaMemsetAsync(c->pr_gamma0, 0, sizeof(float2) * nb, c->st) == cudaSuccess &&
         cudaMemsetAsync(c->pr_state, 0, sizeof(PrtfState) * c->batch, c->st) == cudaSuccess;
    if (!ok) return fail(set_error(CDX_ERR_CUDA, "PRTF buffer clear"));
  }
  if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess)
    return fail(set_error(CDX_ERR_CUDA, "event create failed"));
  if (cudaStreamSynchronize(c->st) != cudaSuccess)
    return fail(set_error(CDX_ERR_CUDA, std::string("context init: ") + cudaGetErrorString(cudaGetLastError())));
  *out = c;
  return CDX_OK;
}

int cdx_destroy(cdx_ctx* c) {
  if (!c) return CDX_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  if (c->weights) cudaFree(c->weights);
  if (c->bs) cudaFree(c->bs);
  if (c->bs_t) cudaFree(c->bs_t);
  if (c->arena) cudaFree(c->arena);
  for (void* q : {(void*)c->pr_psi, (void*)c->pr_rhop, (void*)c->pr_cache, (void*)c->pr_gamma0, (void*)c->pr_map,
                  (void*)c->pr_mask, (void*)c->pr_polar, (void*)c->pr_part, (void*)c->pr_state})
    if (q) cudaFree(q);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->own_stream && c->st) cudaStreamDestroy(c->st);
  delete c;
  return CDX_OK;
}

int cdx_get_prtf(cdx_ctx* c, int idx, float* out, int where) {
  if (!c || !out || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad PRTF argument");
  if (!c->pr_polar || !c->pr_valid) return set_error(CDX_ERR_STATE, "no PRTF: prtf_iter off or not reached");
  const int h = c->rows / 2;
  std::vector<float> w(h), v(h);
  CDX_CK(cudaMemcpyAsync(w.data(), c->pr_polar + (size_t)idx * h, sizeof(float) * h, cudaMemcpyDeviceToHost, c->st));
  CDX_CK(cudaMemcpyAsync(v.data(), c->pr_polar + (size_t)(c->batch + idx) * h, sizeof(float) * h,
                         cudaMemcpyDeviceToHost, c->st));
  CDX_CK(cudaStreamSynchronize(c->st));
  for (int i = 0; i < h; ++i) v[i] = v[i] / w[i];   // prtf[i]/weights[i] (cdi.cc:437-439)
  if (where == CDX_DEVICE) CDX_CK(cudaMemcpy(out, v.data(), sizeof(float) * h, cudaMemcpyHostToDevice));
  else memcpy(out, v.data(), sizeof(float) * h);
  return CDX_OK;
}

int cdx_get_tuning(cdx_ctx* c, int* pdl, int* row_chunk, char* report, int cap) {
  if (!c) return set_error(CDX_ERR_ARG, "null context");
  if (pdl)
    *pdl = (c->tune_pdl_col == 0 && c->tune_pdl_row == 0)
               ? -1
               : (c->tune_pdl_col == 2 ? 1 : 0) | (c->tune_pdl_row == 2 ? 2 : 0);
  if (row_chunk) *row_chunk = c->tune_cb_plus1 - 1;
  if (report && cap > 0) {
    std::strncpy(report, c->tune_report.c_str(), (size_t)cap - 1);
    report[cap - 1] = 0;
  }
  return CDX_OK;
}

int cdx_tuning_save(const char* path) {
  if (!path) return set_error(CDX_ERR_ARG, "null path");
  std::string out = "{\"cdx_tuning\": 1, \"entries\": [";
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    bool first = true;
    for (const auto& kv : g_tune_named) {
      const TuneRec& r = kv.second;
      char line[512];
      snprintf(line, sizeof line,
               "%s\n  {\"device\": \"%s\", \"rows\": %d, \"cols\": %d, \"batch\": %d, \"pdl_col\": %d, "
               "\"pdl_row\": %d, \"row_chunk_bits\": %d, \"us\": %.3f}",
               first ? "" : ",", std::get<0>(kv.first).c_str(), std::get<1>(kv.first), std::get<2>(kv.first),
               std::get<3>(kv.first), r.pdl_col - 1, r.pdl_row - 1, r.cb_plus1 - 1, r.us);
      out += line;
      first = false;
    }
  }
  out += "\n]}\n";
  FILE* f = std::fopen(path, "w");
  if (!f) return set_error(CDX_ERR_IO, std::string("cannot write ") + path);
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  std::fclose(f);
  return ok ? CDX_OK : set_error(CDX_ERR_IO, std::string("short write to ") + path);
}

int cdx_tuning_load(const char* path, int* count) {
  if (!path) return set_error(CDX_ERR_ARG, "null path");
  FILE* f = std::fopen(path, "r");
  if (!f) return set_error(CDX_ERR_IO, std::string("cannot read ") + path);
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  std::fclose(f);
  std::vector<std::pair<std::string, std::pair<std::tuple<int, int, int>, TuneRec>>> entries;
  int e = parse_tuning(text, entries);
  if (e) return e;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  for (const auto& en : entries) {
    const auto& k = en.second.first;
    g_tune_named[std::make_tuple(en.first, std::get<0>(k), std::get<1>(k), std::get<2>(k))] = en.second.second;
    // a decision already made in this process for the same size on a device of that name gives way
    for (auto it = g_tune.begin(); it != g_tune.end();) {
      if (std::get<1>(it->first) == std::get<0>(k) && std::get<2>(it->first) == std::get<1>(k) &&
          std::get<3>(it->first) == std::get<2>(k) && device_name(std::get<0>(it->first)) == en.first)
        it = g_tune.erase(it);
      else
        ++it;
    }
  }
  if (count) *count = (int)entries.size();
  return CDX_OK;
}

int cdx_get_params(const cdx_ctx* c, cdx_params* out) {
  if (!c || !out) return set_error(CDX_ERR_ARG, "null argument");
  *out = c->p;
  return CDX_OK;
}

int cdx_device_arrays(cdx_ctx* c, float** pattern, void** fourier, void** object, float** support) {
  if (!c) return set_error(CDX_ERR_ARG, "null context");
  if (pattern) *pattern = c->inten;
  if (fourier) *fourier = c->psi;
  if (object) *object = c->rho;
  if (support) *support = c->spt;
  return CDX_OK;
}

int cdx_set_pattern(cdx_ctx* c, int idx, const float* inten, int where, int layout, float scale) {
  if (!c || !inten || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad pattern argument");
  const long long off = (long long)idx * c->npx, toff = (long long)idx * c->wstride;
  int e = copy_in(c->inten + off, inten, sizeof(float) * c->npx, where, c->st);
  if (e) return e;
  if (layout == CDX_CENTERED) CDX_CK(convert_fo_real(c->inten + off, c->inten + off, c->rows, c->cols, 1, c->st));
  if (scale != 1.f) CDX_CK(scale_real(c->inten + off, scale, c->npx, c->st));
  CDX_CK(to_tiled(c->inten + off, c->inten_t + toff, c->rows, c->cols, c->tl, c->wstride, 1, c->st));
  CDX_CK(amp_from_pattern(c->inten_t + toff, c->amp_t + toff, c->wstride, c->st));
  CDX_CK(pattern_amp_sum(c->amp_t + toff, c->wstride, 1, c->part, kRedBlocks, c->dstate + idx, c->st));
  CDX_CK(cudaStreamSynchronize(c->st));
  c->have_pattern[idx] = 1;
  return CDX_OK;
}

int cdx_set_beamstop(cdx_ctx* c, int idx, const float* bs, int where, int layout) {
  if (!c || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad beamstop argument");
  if (!bs) return CDX_OK;
  if (!c->bs) {
    CDX_CK(cudaMalloc(&c->bs, sizeof(float) * c->npx * c->batch));
    CDX_CK(cudaMemsetAsync(c->bs, 0, sizeof(float) * c->npx * c->batch, c->st));
    CDX_CK(cudaMalloc(&c->bs_t, sizeof(float) * c->wstride * c->batch));
    CDX_CK(cudaMemsetAsync(c->bs_t, 0, sizeof(float) * c->wstride * c->batch, c->st));
  }
  const long long off = (long long)idx * c->npx, toff = (long long)idx * c->wstride;
  int e = copy_in(c->bs + off, bs, sizeof(float) * c->npx, where, c->st);
  if (e) return e;
  if (layout == CDX_CENTERED) CDX_CK(convert_fo_real(c->bs + off, c->bs + off, c->rows, c->cols, 1, c->st));
  CDX_CK(to_tiled(c->bs + off, c->bs_t + toff, c->rows, c->cols, c->tl, c->wstride, 1, c->st));
  c->gkey.clear();
  CDX_CK(cudaStreamSynchronize(c->st));
  return CDX_OK;
}

// rho0 = IFFT(Psi0) * (1/sqrt(N)) (cdi.cc:225-226); Psi0 stays in psi, where
// the first projection reads it.
static int init_rho_from_psi(cdx_ctx* c, int idx, int count) {
  const long long off = (long long)idx * c->npx;
  const float f = (float)(1.0 / std::sqrt((double)c->rows * c->cols));
  return fft2_enqueue(c->psi + off, c->rho + off, c->rows, c->cols, count, true, f, c->tw_r, c->tw_c, c->st,
                      c->p.fft_mode);
}

int cdx_set_initial(cdx_ctx* c, int idx, const float* psi0, int where) {
  if (!c || !psi0 || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad initial-iterate argument");
  const long long off = (long long)idx * c->npx;
  int e = copy_in(c->psi + off, psi0, sizeof(float2) * c->npx, where, c->st);
  if (e) return e;
  if ((e = init_rho_from_psi(c, idx, 1))) return e;
  if ((e = reset_support(c, idx, 1))) return e;   // initSupport (cdi.cc:227, 252-254)
  CDX_CK(cudaStreamSynchronize(c->st));
  // a batch restarts together: the first iteration reads Psi0 of every pattern
  c->fresh[idx] = 1;
  int nfresh = 0;
  for (char f : c->fresh) nfresh += f;
  c->have_initial = true;
  c->psi_in_work = nfresh == c->batch;
  return CDX_OK;
}

int cdx_random_start(cdx_ctx* c, unsigned long long seed) {
  if (!c) return set_error(CDX_ERR_ARG, "null context");
  for (int i = 0; i < c->batch; ++i)
    if (!c->have_pattern[i]) return set_error(CDX_ERR_STATE, "pattern " + std::to_string(i) + " not set");
  PatState h0;
  CDX_CK(cudaMemcpy(&h0, c->dstate, sizeof h0, cudaMemcpyDeviceToHost));
  CDX_CK(random_start(c->inten, c->bs, h0.threshold, c->psi, c->npx, c->batch, seed, c->st));
  int e = init_rho_from_psi(c, 0, c->batch);
  if (e) return e;
  if ((e = reset_support(c, 0, c->batch))) return e;
  CDX_CK(cudaStreamSynchronize(c->st));
  c->fresh.assign(c->batch, 1);
  c->have_initial = true;
  c->psi_in_work = true;
  return CDX_OK;
}

int cdx_set_support(cdx_ctx* c, int idx, const float* support, int where) {
  if (!c || !support || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad support argument");
  const long long off = (long long)idx * c->npx;
  int e = copy_in(c->spt + off, support, sizeof(float) * c->npx, where, c->st);
  if (e) return e;
  CDX_CK(support_bits(c->spt + off, c->dstate + idx, 0.f, c->mask + (long long)idx * c->rows * c->wpr, c->rows,
                      c->cols, 1, c->st));
  CDX_CK(cudaStreamSynchronize(c->st));
  return CDX_OK;
}

int cdx_set_stop_rfactor(cdx_ctx* c, int idx, double stop) {
  if (!c || idx < 0 || idx >= c->batch || !(stop >= 0.0)) return set_error(CDX_ERR_ARG, "bad stop argument");
  CDX_CK(cudaMemcpyAsync(&c->dstate[idx].stop, &stop, sizeof(double), cudaMemcpyHostToDevice, c->st));
  CDX_CK(cudaStreamSynchronize(c->st));
  return CDX_OK;
}

int cdx_run_async(cdx_ctx* c, const char* algorithm) { return run_impl(c, algorithm); }

int cdx_group_create(cdx_ctx* const* ctxs, int n, cdx_group** out) {
  if (!ctxs || n < 1 || !out) return set_error(CDX_ERR_ARG, "bad group argument");
  *out = nullptr;
  cdx_group* g = new cdx_group();
  for (int i = 0; i < n; ++i) {
    if (!ctxs[i]) { delete g; return set_error(CDX_ERR_ARG, "null context in group"); }
    for (cdx_ctx* o : g->ctxs)
      if (o->st == ctxs[i]->st) { delete g; return set_error(CDX_ERR_ARG, "group contexts must use distinct streams"); }
    g->ctxs.push_back(ctxs[i]);
  }
  bool ok = cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreate(&g->ev0) == cudaSuccess && cudaEventCreate(&g->ev1) == cudaSuccess;
  g->joins.assign(n, nullptr);
  for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&g->joins[i], cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    cdx_group_destroy(g);
    return set_error(CDX_ERR_CUDA, "group stream/event creation failed");
  }
  *out = g;
  return CDX_OK;
}

int cdx_group_run(cdx_group* g, const char* algorithm, double* gpu_ms) {
  if (!g) return set_error(CDX_ERR_ARG, "null group");
  return group_run_impl(g, algorithm, gpu_ms);
}

int cdx_group_set_concurrent(cdx_group* g, int concurrent) {
  if (!g) return set_error(CDX_ERR_ARG, "null group");
  g->concurrent = concurrent != 0;
  return CDX_OK;
}

int cdx_group_destroy(cdx_group* g) {
  if (!g) return CDX_OK;
  if (g->st) cudaStreamSynchronize(g->st);
  if (g->gexec) cudaGraphExecDestroy(g->gexec);
  for (cudaEvent_t e : g->joins)
    if (e) cudaEventDestroy(e);
  if (g->fork) cudaEventDestroy(g->fork);
  if (g->ev0) cudaEventDestroy(g->ev0);
  if (g->ev1) cudaEventDestroy(g->ev1);
  if (g->st) cudaStreamDestroy(g->st);
  delete g;
  return CDX_OK;
}

// A pass kernel whose staging copy did not complete within its bounded wait
// leaves bit 0 in the context's error word; reported (and cleared) here.
int check_bulk(cdx_ctx* c) {
  int h = 0;
  CDX_CK(cudaMemcpy(&h, c->derr, sizeof(int), cudaMemcpyDeviceToHost));
  if (h) {
    CDX_CK(cudaMemset(c->derr, 0, sizeof(int)));
    return set_error(CDX_ERR_CUDA, "a pass kernel's bulk staging copy timed out; the run's results are invalid");
  }
  return CDX_OK;
}

int cdx_run(cdx_ctx* c, const char* algorithm, cdx_stats* stats) {
  int e = run_impl(c, algorithm);
  if (e) return e;
  CDX_CK(cudaStreamSynchronize(c->st));
  if ((e = check_bulk(c))) return e;
  return fill_stats(c, 0, stats);
}

int cdx_get_stats(cdx_ctx* c, int idx, cdx_stats* s) {
  if (!c || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad stats argument");
  return fill_stats(c, idx, s);
}

int cdx_get_object(cdx_ctx* c, int idx, float* out, int where) {
  if (!c || !out || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad output argument");
  return copy_out(out, c->rho + (long long)idx * c->npx, sizeof(float2) * c->npx, where, c->st);
}
int cdx_get_fourier(cdx_ctx* c, int idx, float* out, int where) {
  if (!c || !out || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad output argument");
  return copy_out(out, c->psi + (long long)idx * c->npx, sizeof(float2) * c->npx, where, c->st);
}
int cdx_get_support(cdx_ctx* c, int idx, float* out, int where) {
  if (!c || !out || idx < 0 || idx >= c->batch) return set_error(CDX_ERR_ARG, "bad output argument");
  return copy_out(out, c->spt + (long long)idx * c->npx, sizeof(float) * c->npx, where, c->st);
}

namespace {

// cdx_phase_retrieve_host keeps the context of its last call (device arrays and
// the CUDA graph of the last algorithm) for the next call with the same
// parameters on the same device, as the reference keeps its memory pool and its
// cuFFT plan for the whole process (memManager.cc, cudaConfig.cu:137-159).
struct HostSlot {
  cdx_ctx* ctx = nullptr;
  cdx_params key{};
  int device = -1;
  bool busy = false;
};
std::mutex g_host_mu;
HostSlot g_host_slot;

// Return a kept context to the state cdx_create leaves: arena zeroed,
// vars.threshold 0.5, rect support, no pattern or initial iterate set.
int ctx_reset(cdx_ctx* c) {
  CDX_CK(cudaSetDevice(c->device));
  CDX_CK(cudaMemsetAsync(c->arena, 0, c->arena_bytes, c->st));
  CDX_CK(state_init(c->dstate, c->batch, 0.5f, c->st));
  int e = reset_support(c, 0, c->batch);
  if (e) return e;
  if (c->pr_cache) {
    const size_t nb = (size_t)c->batch * c->npx;
    CDX_CK(cudaMemsetAsync(c->pr_cache, 0, sizeof(float2) * nb, c->st));
    CDX_CK(cudaMemsetAsync(c->pr_gamma0, 0, sizeof(float2) * nb, c->st));
    CDX_CK(cudaMemsetAsync(c->pr_state, 0, sizeof(PrtfState) * c->batch, c->st));
  }
  c->have_pattern.assign(c->batch, 0);
  c->fresh.assign(c->batch, 0);
  c->have_initial = false;
  c->psi_in_work = false;
  c->pr_valid = false;
  CDX_CK(cudaStreamSynchronize(c->st));
  return CDX_OK;
}

}  // namespace

int cdx_phase_retrieve_host(const cdx_params* p, const char* algorithm, const float* inten, const float* psi0,
                            unsigned long long seed, float* rho_out, float* psi_out, float* support_out,
                            cdx_stats* stats) {
  if (!p || !inten) return set_error(CDX_ERR_ARG, "null argument");
  cdx_params q = *p;
  q.batch = 1;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(CDX_ERR_NOLIB, "no CUDA device");
  cdx_ctx* c = nullptr;
  bool kept = false;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    if (g_host_slot.ctx && !g_host_slot.busy && g_host_slot.device == dev &&
        std::memcmp(&g_host_slot.key, &q, sizeof q) == 0) {
      c = g_host_slot.ctx;
      g_host_slot.busy = true;
      kept = true;
    }
  }
  int e = kept ? ctx_reset(c) : cdx_create(&q, nullptr, &c);
  if (e && !kept) return e;
  if (e) goto done;
  if ((e = cdx_set_pattern(c, 0, inten, CDX_HOST, CDX_FFT_ORDER, 1.f))) goto done;
  e = psi0 ? cdx_set_initial(c, 0, psi0, CDX_HOST) : cdx_random_start(c, seed);
  if (e) goto done;
  if ((e = cdx_run(c, algorithm, stats))) goto done;
  if (rho_out && (e = cdx_get_object(c, 0, rho_out, CDX_HOST))) goto done;
  if (psi_out && (e = cdx_get_fourier(c, 0, psi_out, CDX_HOST))) goto done;
  if (support_out && (e = cdx_get_support(c, 0, support_out, CDX_HOST))) goto done;
done:
  {
    std::unique_lock<std::mutex> lk(g_host_mu);
    if (kept) {
      if (e) g_host_slot = HostSlot{};   // a context that failed is not kept
      else {
        g_host_slot.busy = false;
        c = nullptr;
      }
    } else if (!e && !g_host_slot.ctx) {
      g_host_slot.ctx = c;
      g_host_slot.key = q;
      g_host_slot.device = dev;
      g_host_slot.busy = false;
      c = nullptr;
    }
  }
  if (c) cdx_destroy(c);
  return e;
}

int cdx_release_host_cache(void) {
  cdx_ctx* c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_host_mu);
    if (g_host_slot.busy) return set_error(CDX_ERR_STATE, "the kept context is in use by a running call");
    c = g_host_slot.ctx;
    g_host_slot = HostSlot{};
  }
  return c ? cdx_destroy(c) : CDX_OK;
}

// ---------------------------------------------------------------- primitives
int cdx_fft2(const void* in, void* out, int rows, int cols, int batch, int inverse, void* stream) {
  return cdx_fft2_ex(in, out, rows, cols, batch, inverse, CDX_FFT_FP32, stream);
}

int cdx_fft2_ex(const void* in, void* out, int rows, int cols, int batch, int inverse, int fft_mode, void* stream) {
  if (!in || !out || batch < 1) return set_error(CDX_ERR_ARG, "bad fft argument");
  if (fft_mode != CDX_FFT_FP32 && fft_mode != CDX_FFT_TC_BF16 && fft_mode != CDX_FFT_TC_MMA)
    return set_error(CDX_ERR_ARG, "unknown fft_mode");
  int e = check_len(rows);
  if (e) return e;
  if ((e = check_len(cols))) return e;
  if (prep_launcher(rows)() != cudaSuccess || prep_launcher(cols)() != cudaSuccess)
    return set_error(CDX_ERR_CUDA, "kernel attributes");
  float2 *tr, *tc;
  if ((e = twiddles(rows, &tr)) || (e = twiddles(cols, &tc))) return e;
  return fft2_enqueue((const float2*)in, (float2*)out, rows, cols, batch, inverse != 0, 1.f, tr, tc,
                      (cudaStream_t)stream, fft_mode);
}

int cdx_apply_mod_abs(void* psi, const float* inten, long long n, void* stream) {
  if (!psi || !inten || n < 0) return set_error(CDX_ERR_ARG, "bad argument");
  CDX_CK(mod_abs((float2*)psi, inten, n, (cudaStream_t)stream));
  return CDX_OK;
}

int cdx_apply_mod(void* psi, const float* inten, const float* bs, int noise, float scale, int rcolor, long long n,
                  void* stream) {
  if (!psi || !inten || n < 0 || rcolor == 0 || scale == 0) return set_error(CDX_ERR_ARG, "bad argument");
  CDX_CK(mod_ccd((float2*)psi, inten, bs, noise, scale, (float)rcolor, n, (cudaStream_t)stream));
  return CDX_OK;
}

int cdx_apply_support(void* rho, const void* rhop, const float* spt, float thr, float beta, int algo, long long n,
                      void* stream) {
  if (!rho || !rhop || !spt || n < 0) return set_error(CDX_ERR_ARG, "bad argument");
  CDX_CK(apply_support((float2*)rho, (const float2*)rhop, spt, thr, beta, algo, n, (cudaStream_t)stream));
  return CDX_OK;
}

int cdx_convert_fo(const void* in, void* out, int rows, int cols, int batch, int is_complex, void* stream) {
  if (!in || !out || rows < 2 || cols < 2 || batch < 1 || rows % 2 || cols % 2)
    return set_error(CDX_ERR_ARG, "bad argument");
  if (in != out && is_complex)
    CDX_CK(cudaMemcpyAsync(out, in, sizeof(float2) * rows * cols * batch, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  if (in != out && !is_complex)
    CDX_CK(cudaMemcpyAsync(out, in, sizeof(float) * rows * cols * batch, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  if (is_complex) CDX_CK(convert_fo_complex((const float2*)out, (float2*)out, rows, cols, batch, (cudaStream_t)stream));
  else CDX_CK(convert_fo_real((const float*)out, (float*)out, rows, cols, batch, (cudaStream_t)stream));
  return CDX_OK;
}

int cdx_algo_expand(const char* algorithm, int* out, int cap, int* count) {
  std::vector<int> v;
  int e = algo_expand(algorithm, v, 50000000);
  if (e) return e;
  if (count) *count = (int)v.size();
  if (out)
    for (int i = 0; i < (int)v.size() && i < cap; ++i) out[i] = v[i];
  return CDX_OK;
}

int cdx_read_bin(const char* path, int* rows, int* cols, int* is_complex, float* data, size_t cap) {
  if (!path || !rows || !cols || !is_complex) return set_error(CDX_ERR_ARG, "null argument");
  return read_bin(path, rows, cols, is_complex, data, cap);
}
int cdx_write_bin(const char* path, const float* data, int rows, int cols, int is_complex) {
  if (!path || !data || rows <= 0 || cols <= 0) return set_error(CDX_ERR_ARG, "bad argument");
  return write_bin(path, data, rows, cols, is_complex);
}

}  // extern "C"
