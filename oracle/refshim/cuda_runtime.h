// Host stand-ins for the CUDA runtime calls the reference hot path makes:
// device memory is host memory, copies are memcpy.
#pragma once
#include "cdxref_host.h"
typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice,
                      cudaMemcpyDefault };
typedef void* cudaStream_t;
inline const char* cudaGetErrorString(int) { return "cuda error (host emulation)"; }
// sizes rounded up to 512 bytes like the device allocator's blocks: the reference's
// regularize_zernike_coefficients (beamDecomposition.cu:480-513) touches its whole
// last thread block of modes, past the coefficients' end but inside that rounding
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = calloc((n + 511) / 512 * 512 + (n ? 0 : 512), 1); return *p ? 0 : 2; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
inline cudaError_t cudaFree(void* p) { free(p); return 0; }
inline cudaError_t cudaMemset(void* p, int v, size_t n) { memset(p, v, n); return 0; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return 0; }
inline cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind, cudaStream_t = 0) {
  memmove(d, s, n); return 0; }
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0, cudaMemcpyKind = cudaMemcpyHostToDevice) {
  memcpy((char*)&sym + off, src, n); return 0; }
template <class T>
inline cudaError_t cudaMemcpyFromSymbol(void* dst, const T& sym, size_t n, size_t off = 0, cudaMemcpyKind = cudaMemcpyDeviceToHost) {
  memcpy(dst, (const char*)&sym + off, n); return 0; }
inline cudaError_t cudaGetLastError() { return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
inline cudaError_t cudaMemGetInfo(size_t* f, size_t* t) { *f = *t = (size_t)1 << 40; return 0; }
inline cudaError_t cudaSetDevice(int) { return 0; }
inline cudaError_t cudaGetDevice(int* d) { *d = 0; return 0; }
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct double2 { double x, y; };
struct int2 { int x, y; };
struct uchar3 { unsigned char x, y, z; };
inline float2 make_float2(float a, float b) { return {a, b}; }
inline double2 make_double2(double a, double b) { return {a, b}; }
inline float3 make_float3(float a, float b, float c) { return {a, b, c}; }
inline float4 make_float4(float a, float b, float c, float d) { return {a, b, c, d}; }
