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
// Scratch layout (g_noalloc_scratch; rows x cols pattern, L = column-pass
// lines per CTA of length `rows`, cp = cols padded to L):
//   twiddle tables of every supported length   written once per device at set-up
//   error word                                  cleared by every call
//   column-tiled work buffer   rows*cp complex  cleared by every call
//   column-tiled sqrt(I)       rows*cp float
//   support bits               rows*ceil(cols/32) words
// Every call shares the array and it keeps the last call's contents: each
// call clears the regions it uses before use, and calls that overlap on the
// GPU (two streams, two host threads) race on it.  The first call on a device
// is its set-up: it looks up the array's device address there
// (cudaGetSymbolAddress) and copies the twiddle tables in with a blocking
// cudaMemcpy; make that first call outside any stream capture.  Later calls
// only queue a memset and kernels on the caller's stream and return.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/cdx.h"
#include "cdx_fft.cuh"
#include "cdx_host.h"
#include "cdx_misc.h"
#include "cdx_types.h"

using namespace cdx;

static __device__ __align__(256) unsigned char g_noalloc_scratch[CDX_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
// the lengths the pass kernels support (cdx_size_supported), in table order
constexpr int kLens[] = {16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096};
constexpr int kNumLens = (int)(sizeof(kLens) / sizeof(kLens[0]));

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

std::mutex g_mu;
void* g_addr[kMaxDevices];   // device address of g_noalloc_scratch per device (nullptr: not set up)
size_t g_tw_off[kNumLens];   // byte offset of each length's twiddle table in the scratch
size_t g_tw_bytes;           // bytes of all twiddle tables (start of the per-call region)

int len_index(int n) {
  for (int i = 0; i < kNumLens; ++i)
    if (kLens[i] == n) return i;
  return -1;
}

// Host code only sees a stand-in for the array; its device address comes from
// cudaGetSymbolAddress, once per device, with that device current.  The same
// set-up copies the per-pass twiddle tables of every length (the context
// path's tables, cdx_dispatch.cu) to the front of the array; they are never
// written again, so later calls need no host-to-device copy.
int scratch_setup(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error_cstr(CDX_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error_cstr(CDX_ERR_ARG, "device ordinal beyond the supported range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    if (!g_tw_bytes) {
      size_t off = 0;
      for (int i = 0; i < kNumLens; ++i) {
        g_tw_off[i] = off;
        off += al256(sizeof(float2) * (size_t)(twiddle_count(kLens[i]) > 0 ? twiddle_count(kLens[i]) : 1));
      }
      g_tw_bytes = off;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      char msg[256];
      snprintf(msg, sizeof msg, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
      return set_error_cstr(CDX_ERR_CUDA, msg);
    }
    std::vector<float2> host(g_tw_bytes / sizeof(float2), make_float2(0.f, 0.f));
    for (int i = 0; i < kNumLens; ++i)
      if (twiddle_count(kLens[i]) > 0) twiddle_table(kLens[i], host.data() + g_tw_off[i] / sizeof(float2));
    e = cudaMemcpy(p, host.data(), g_tw_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      char msg[256];
      snprintf(msg, sizeof msg, "twiddle set-up copy: %s", cudaGetErrorString(e));
      return set_error_cstr(CDX_ERR_CUDA, msg);
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return CDX_OK;
}

// The closing step of a call: rho *= sqrt(N) (applyNorm at the end of
// phaseRetrieve, cdi.cc:406).  A staging wait of a pass kernel that ran out
// (bit 0 of *err; it guards against a hang and has not been seen) leaves the
// results invalid, and the call has already returned: both outputs become NaN
// so the caller cannot take them for a result.
__global__ void k_noalloc_finish(float2* rho, float2* psi, float s, long long n, const int* err) {
  const bool bad = *err != 0;
  const float nan = __int_as_float(0x7fc00000);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    float2 v = rho[i];
    rho[i] = bad ? make_float2(nan, nan) : make_float2(v.x * s, v.y * s);
    if (bad) psi[i] = make_float2(nan, nan);
  }
}

bool overlap(const void* a, size_t na, const void* b, size_t nb) {
  const char* pa = (const char*)a;
  const char* pb = (const char*)b;
  return pa < pb + nb && pb < pa + na;
}

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
  const long long npx = (long long)rows * cols;
  // the pass kernels stage rows and columns by 16-byte copies
  for (const void* q : {(const void*)intensity, (const void*)support, psi0, (const void*)rho_out, (const void*)psi_out})
    if ((uintptr_t)q % 16)
      return set_error_cstr(CDX_ERR_ARG, "cdx_iterate_noalloc: every buffer must start on a 16-byte boundary");
  // rho_out is written before Psi0 is read for the last time; the outputs must
  // not alias each other or the inputs (psi_out == psi0 exactly is allowed)
  const size_t bf = sizeof(float) * npx, bc = sizeof(float2) * npx;
  if (overlap(rho_out, bc, intensity, bf) || overlap(rho_out, bc, support, bf) || overlap(rho_out, bc, psi0, bc) ||
      overlap(rho_out, bc, psi_out, bc) || overlap(psi_out, bc, intensity, bf) || overlap(psi_out, bc, support, bf) ||
      (psi_out != psi0 && overlap(psi_out, bc, psi0, bc)))
    return set_error_cstr(CDX_ERR_ARG, "cdx_iterate_noalloc: rho_out/psi_out overlap another buffer");
  const int lc = lines_per_cta(rows);
  int tl = 0;
  while ((1 << tl) < lc) ++tl;
  const long long cp = ((long long)cols + lc - 1) / lc * lc;
  const long long wst = (long long)rows * cp;
  const int wpr = (cols + 31) >> 5;

  void* base = nullptr;
  int e = scratch_setup(&base);
  if (e) return e;
  const size_t o_err = g_tw_bytes;
  const size_t o_work = o_err + 256;
  const size_t o_amp = o_work + al256(sizeof(float2) * wst);
  const size_t o_mask = o_amp + al256(sizeof(float) * wst);
  const size_t need = o_mask + al256(sizeof(uint32_t) * rows * wpr);
  if (need > CDX_NOALLOC_SCRATCH_BYTES)
    return set_error_cstr(CDX_ERR_SIZE, "cdx_iterate_noalloc: pattern needs more scratch than the static array holds");
  cudaStream_t st = (cudaStream_t)stream;
  if (prep_launcher(rows)() != cudaSuccess || prep_launcher(cols)() != cudaSuccess)
    return set_error_cstr(CDX_ERR_CUDA, "cdx_iterate_noalloc: kernel attributes");
  char* s = (char*)base;
  int* err = (int*)(s + o_err);
  float2* work = (float2*)(s + o_work);
  float* amp_t = (float*)(s + o_amp);
  uint32_t* mask = (uint32_t*)(s + o_mask);
  const float2* tw_r = (const float2*)(s + g_tw_off[len_index(rows)]);
  const float2* tw_c = (const float2*)(s + g_tw_off[len_index(cols)]);

  // the array keeps the previous call's contents: clear what this call uses
  NA_CK(cudaMemsetAsync(s + o_err, 0, need - o_err, st));
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
    r.err = err;
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
    c.err = err;
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
    c.err = err;
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
    r.err = err;
    NA_CK(row_launcher(cols)(r, 1, st));
  }
  // Psi = FFT(rho) (the last myFFT), or Psi0 when no iteration ran
  if (iterations == 0) {
    if (psi_out != psi0) NA_CK(cudaMemcpyAsync(psi_out, psi0, sizeof(float2) * npx, cudaMemcpyDeviceToDevice, st));
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
    c.err = err;
    NA_CK(col_launcher(rows)(c, 1, st));
  }
  // applyNorm(rho, sqrt(N)) at the end of phaseRetrieve (cdi.cc:406), or NaN
  // outputs if a staging wait ran out
  const int blocks = (int)std::min<long long>((npx + 255) / 256, 1024);
  k_noalloc_finish<<<blocks, 256, 0, st>>>(rho, (float2*)psi_out, (float)std::sqrt((double)npx), npx, err);
  NA_CK(cudaGetLastError());
  return CDX_OK;
}
