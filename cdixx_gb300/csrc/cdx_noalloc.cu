// cdx_iterate_noalloc: the fused iteration (column pass + row pass) for
// callers that cannot allocate device memory.
//
// Who needs it: a detector's acquisition loop that cannot afford the implicit
// device-wide synchronisation of cudaMalloc/cudaFree between frames, and a
// plugin hosted by an application that owns the whole device-memory budget
// and forbids private allocations.  Such a caller hands in its own device
// buffers for the inputs (pattern, support, restart iterate) and outputs
// (rho, Psi); everything else the kernels need lives in one file-scope
// __device__ array of this library, present on every GPU that loads the
// library until the process exits.
//
// Scratch layout (carved per call from g_noalloc_scratch, rows x cols pattern,
// L = column-pass lines per CTA of length `rows`, cp = cols padded to L):
//   column-tiled work buffer   rows*cp complex
//   column-tiled sqrt(I)       rows*cp float
//   support bits               rows*ceil(cols/32) words
//   twiddles of rows and cols  per-pass tables
// Every call shares the array and it keeps the last call's contents: each
// call clears the regions it uses before use, and calls that overlap on the
// GPU (two streams, two host threads) race on it.  The first call on a device
// looks up the array's device address there (cudaGetSymbolAddress); make
// that first call outside any stream capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "../../include/cdx.h"
#include "cdx_fft.cuh"
#include "cdx_host.h"
#include "cdx_misc.h"
#include "cdx_types.h"

using namespace cdx;

static __device__ __align__(256) unsigned char g_noalloc_scratch[CDX_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices];   // device address of g_noalloc_scratch per device (nullptr: not looked up)

// Host code only sees a stand-in for the array; its device address comes from
// cudaGetSymbolAddress, once per device, with that device current.
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error_cstr(CDX_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error_cstr(CDX_ERR_ARG, "device ordinal beyond the supported range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      char msg[256];
      snprintf(msg, sizeof msg, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      return set_error_cstr(CDX_ERR_CUDA, msg);
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return CDX_OK;
}

// Per-pass twiddle tables, filled on the host by the same routine as the
// context path's (cdx_dispatch.cu), so both entry points use identical
// values.  Static host storage (the largest table, length 4096, has 8160
// entries); a call copies its tables from there into the device scratch.
constexpr int kMaxTw = 8192;
static float2 g_tw_host[2][kMaxTw];

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

#define NA_CK(call)                                                                            \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) {                                                                   \
      char m_[256];                                                                            \
      snprintf(m_, sizeof m_, "%s: %s", #call, cudaGetErrorString(e_));                        \
      return set_error_cstr(CDX_ERR_CUDA, m_);                                                 \
    }                                                                                          \
  } while (0)

}  // namespace

extern "C" int cdx_iterate_noalloc(int rows, int cols, int algo, float beta, int iterations, const float* intensity,
                                   const float* support, float threshold, const void* psi0, void* rho_out,
                                   void* psi_out, void* stream) {
  if (!intensity || !support || !psi0 || !rho_out || !psi_out || iterations < 0)
    return set_error_cstr(CDX_ERR_ARG, "cdx_iterate_noalloc: null buffer or negative iteration count");
  if (!cdx_size_supported(rows) || !cdx_size_supported(cols) || rows % 2 || cols % 2)
    return set_error_cstr(CDX_ERR_SIZE, "cdx_iterate_noalloc: rows and cols must be even 2^a 3^b in [16, 4096]");
  if ((long long)rows * cols > CDX_NOALLOC_MAX_PIXELS)
    return set_error_cstr(CDX_ERR_SIZE, "cdx_iterate_noalloc: pattern larger than CDX_NOALLOC_MAX_PIXELS");
  if (algo < CDX_RAAR || algo > CDX_KKT || algo == CDX_SHRINKWRAP)
    return set_error_cstr(CDX_ERR_ALGO, "cdx_iterate_noalloc: algo must be a real-space update (no shrinkWrap/TV)");
  const int lc = lines_per_cta(rows);
  int tl = 0;
  while ((1 << tl) < lc) ++tl;
  const long long cp = ((long long)cols + lc - 1) / lc * lc;
  const long long wst = (long long)rows * cp;
  const int wpr = (cols + 31) >> 5;
  const int ntr = twiddle_count(rows), ntc = twiddle_count(cols);
  if (ntr > kMaxTw || ntc > kMaxTw) return set_error_cstr(CDX_ERR_SIZE, "cdx_iterate_noalloc: twiddle table too long");
  const size_t o_work = 0;
  const size_t o_amp = o_work + al256(sizeof(float2) * wst);
  const size_t o_mask = o_amp + al256(sizeof(float) * wst);
  const size_t o_twr = o_mask + al256(sizeof(uint32_t) * rows * wpr);
  const size_t o_twc = o_twr + al256(sizeof(float2) * (ntr > 0 ? ntr : 1));
  const size_t need = o_twc + al256(sizeof(float2) * (ntc > 0 ? ntc : 1));
  if (need > CDX_NOALLOC_SCRATCH_BYTES)
    return set_error_cstr(CDX_ERR_SIZE, "cdx_iterate_noalloc: pattern needs more scratch than the static array holds");

  void* base = nullptr;
  int e = scratch_address(&base);
  if (e) return e;
  cudaStream_t st = (cudaStream_t)stream;
  if (prep_launcher(rows)() != cudaSuccess || prep_launcher(cols)() != cudaSuccess)
    return set_error_cstr(CDX_ERR_CUDA, "cdx_iterate_noalloc: kernel attributes");
  char* s = (char*)base;
  float2* work = (float2*)(s + o_work);
  float* amp_t = (float*)(s + o_amp);
  uint32_t* mask = (uint32_t*)(s + o_mask);
  float2* tw_r = (float2*)(s + o_twr);
  float2* tw_c = (float2*)(s + o_twc);
  const long long npx = (long long)rows * cols;

  // the array keeps the previous call's contents: clear what this call uses
  NA_CK(cudaMemsetAsync(s, 0, need, st));
  {
    // the host tables are shared by all calls: fill and copy under the lock
    static std::mutex tw_lock;
    std::lock_guard<std::mutex> g(tw_lock);
    if (ntr > 0) {
      twiddle_table(rows, g_tw_host[0]);
      NA_CK(cudaMemcpyAsync(tw_r, g_tw_host[0], sizeof(float2) * ntr, cudaMemcpyHostToDevice, st));
    }
    if (ntc > 0) {
      twiddle_table(cols, g_tw_host[1]);
      NA_CK(cudaMemcpyAsync(tw_c, g_tw_host[1], sizeof(float2) * ntc, cudaMemcpyHostToDevice, st));
    }
    NA_CK(cudaStreamSynchronize(st));   // the host tables may be refilled by the next call
  }
  // sqrt(I), column-tiled (applyModAbs's sqrtf of I > 0, else 0)
  NA_CK(to_tiled(intensity, amp_t, rows, cols, tl, wst, 1, st));
  NA_CK(amp_from_pattern(amp_t, amp_t, wst, st));
  // support bits: support > threshold (the test of cdi.cu:525)
  NA_CK(support_bits(support, nullptr, threshold, mask, rows, cols, 1, st));

  // rho0 = IFFT(Psi0)/sqrt(N) (prepareIter, cdi.cc:225-226), then the
  // 1/sqrt(N) at the start of phaseRetrieve (cdi.cc:313); rho_out holds rho
  const float isq = (float)(1.0 / std::sqrt((double)npx));
  float2* rho = (float2*)rho_out;
  {
    RowArgs r{};
    r.in = (const float2*)psi0;
    r.out = rho;
    r.in_stride = r.out_stride = npx;
    r.tw = tw_c;
    r.rows = rows;
    r.mode = ROW_FFT;
    r.inv = 1;
    r.scale = 1.f;
    NA_CK(row_launcher(cols)(r, 1, st));
    ColArgs c{};
    c.in = rho;
    c.out = rho;
    c.in_stride = c.out_stride = npx;
    c.tw = tw_r;
    c.cols = cols;
    c.mode = COL_FFT;
    c.inv = 1;
    c.scale = isq;
    NA_CK(col_launcher(rows)(c, 1, st));
  }
  NA_CK(scale_complex(rho, isq, npx, st));

  for (int it = 0; it < iterations; ++it) {
    ColArgs c{};
    const bool first = it == 0;
    c.in = first ? (const float2*)psi0 : work;   // the first projection reads Psi0 itself
    c.in_tiled = first ? 0 : 1;
    c.in_stride = first ? npx : wst;
    c.out = work;
    c.out_tiled = 1;
    c.out_stride = wst;
    c.amp = amp_t;
    c.aux_stride = wst;
    c.tw = tw_r;
    c.cols = cols;
    c.mode = COL_ITER;
    c.from_psi = first;
    c.proj = PROJ_MODABS;
    c.scale = 1.f;
    NA_CK(col_launcher(rows)(c, 1, st));
    RowArgs r{};
    r.in = work;
    r.out = work;
    r.in_tiled = r.out_tiled = 1;
    r.tile_log2 = tl;
    r.in_stride = r.out_stride = wst;
    r.rho = rho;
    r.rho_stride = npx;
    r.mask = mask;
    r.mask_stride = (long long)rows * wpr;
    r.tw = tw_c;
    r.rows = rows;
    r.mode = ROW_ITER;
    r.algo = algo;
    r.scale = 1.f;
    r.inv_n = (float)(1.0 / ((double)rows * cols));
    r.beta = beta;
    NA_CK(row_launcher(cols)(r, 1, st));
  }
  // Psi = FFT(rho) (the last myFFT), or Psi0 when no iteration ran
  if (iterations == 0) {
    NA_CK(cudaMemcpyAsync(psi_out, psi0, sizeof(float2) * npx, cudaMemcpyDeviceToDevice, st));
  } else {
    ColArgs c{};
    c.in = work;
    c.in_tiled = 1;
    c.in_stride = wst;
    c.out = (float2*)psi_out;
    c.out_tiled = 0;
    c.out_stride = npx;
    c.tw = tw_r;
    c.cols = cols;
    c.mode = COL_FFT;
    c.scale = 1.f;
    NA_CK(col_launcher(rows)(c, 1, st));
  }
  // applyNorm(rho, sqrt(N)) at the end of phaseRetrieve (cdi.cc:406)
  NA_CK(scale_complex(rho, (float)std::sqrt((double)npx), npx, st));
  return CDX_OK;
}
