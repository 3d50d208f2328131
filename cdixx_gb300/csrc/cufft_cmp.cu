// Bench-only comparator (never part of the product path or libcdx.so): one
// CDI iteration with the reference's structure -- cuFFT C2C transforms and one
// element-wise kernel per operation, on the default stream order of
// CDI::phaseRetrieve (src/post_gpu/cdi.cc:349-381):
//   applyModAbs(Psi, I)          cudaConfig.cu:827-841
//   myIFFT(Psi, rho')            cudaConfig.cu:175-180 (cufftExecC2C inverse)
//   applyNorm(rho', 1/N)         cudaConfig.cu:425-429
//   ApplyHIOSupport(rho, rho')   cdi.cu:518-533 (float support, threshold)
//   myFFT(rho, Psi)              cudaConfig.cu:175-180 (cufftExecC2C forward)
// The kernels are written here from those definitions; the point is to time
// the reference's launch and memory-traffic structure on the same GPU as the
// fused two-kernel iteration.  Built into _lib/libcdx_cufft_cmp.so by
// cdixx_gb300/build.py, loaded only by bench.py's comparator section.
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdio>

namespace {

__global__ void k_mod_abs(float2* __restrict__ psi, const float* __restrict__ inten, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float I = inten[i];
    const float a = I > 0.f ? sqrtf(I) : 0.f;
    float2 v = psi[i];
    const float m = hypotf(v.x, v.y);
    psi[i] = m == 0.f ? make_float2(a, 0.f) : make_float2(v.x * a / m, v.y * a / m);
  }
}

__global__ void k_norm(float2* __restrict__ x, float s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 v = x[i];
    x[i] = make_float2(v.x * s, v.y * s);
  }
}

__global__ void k_hio(float2* __restrict__ rho, const float2* __restrict__ rhop, const float* __restrict__ spt,
                      float thr, float beta, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float2 p = rhop[i];
    if (spt[i] > thr) {
      rho[i] = p;
    } else {
      const float2 r = rho[i];
      rho[i] = make_float2(r.x - beta * p.x, r.y - beta * p.y);
    }
  }
}

struct Plan {
  cufftHandle h = 0;
  int rows = 0, cols = 0, batch = 0;
  cudaStream_t st = nullptr;
};
Plan g_plan;

}  // namespace

extern "C" {

// Enqueue `iters` reference-structure HIO iterations on `stream` for `batch`
// row-major rows x cols patterns (device buffers): psi (Fourier iterate, in and
// out), rho (object iterate), rhop (scratch, complex), inten (I), spt (float
// support).  Returns 0, or a cuFFT / CUDA error code.
int cmp_iterate(int rows, int cols, int batch, int iters, void* psi, void* rho, void* rhop, const float* inten,
                const float* spt, float thr, float beta, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (!g_plan.h || g_plan.rows != rows || g_plan.cols != cols || g_plan.batch != batch) {
    if (g_plan.h) cufftDestroy(g_plan.h);
    g_plan = Plan{};
    int dims[2] = {rows, cols};
    if (cufftPlanMany(&g_plan.h, 2, dims, nullptr, 1, rows * cols, nullptr, 1, rows * cols, CUFFT_C2C, batch) !=
        CUFFT_SUCCESS)
      return 1001;
    g_plan.rows = rows;
    g_plan.cols = cols;
    g_plan.batch = batch;
  }
  if (cufftSetStream(g_plan.h, st) != CUFFT_SUCCESS) return 1002;
  const long long n = (long long)rows * cols * batch;
  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = (int)((n + 255) / 256 < (long long)sms * 16 ? (n + 255) / 256 : (long long)sms * 16);
  const float inv_n = 1.f / ((float)rows * cols);
  cufftComplex* P = (cufftComplex*)psi;
  cufftComplex* R = (cufftComplex*)rho;
  cufftComplex* Q = (cufftComplex*)rhop;
  for (int it = 0; it < iters; ++it) {
    k_mod_abs<<<blocks, 256, 0, st>>>((float2*)P, inten, n);
    if (cufftExecC2C(g_plan.h, P, Q, CUFFT_INVERSE) != CUFFT_SUCCESS) return 1003;
    k_norm<<<blocks, 256, 0, st>>>((float2*)Q, inv_n, n);
    k_hio<<<blocks, 256, 0, st>>>((float2*)R, (const float2*)Q, spt, thr, beta, n);
    if (cufftExecC2C(g_plan.h, R, P, CUFFT_FORWARD) != CUFFT_SUCCESS) return 1004;
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? 0 : (int)e;
}

}  // extern "C"
