#pragma once
#include "cuda_runtime.h"
typedef float2 cuFloatComplex;
typedef double2 cuDoubleComplex;
inline float cuCrealf(float2 a) { return a.x; }
inline float cuCimagf(float2 a) { return a.y; }
inline float2 make_cuComplex(float a, float b) { return {a, b}; }
inline float2 make_cuFloatComplex(float a, float b) { return {a, b}; }
inline float2 cuConjf(float2 a) { return {a.x, -a.y}; }
inline float2 cuCaddf(float2 a, float2 b) { return {a.x + b.x, a.y + b.y}; }
inline float2 cuCsubf(float2 a, float2 b) { return {a.x - b.x, a.y - b.y}; }
inline float2 cuCmulf(float2 a, float2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
inline float2 cuCdivf(float2 a, float2 b) {
  float d = b.x * b.x + b.y * b.y; return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d}; }
inline float cuCabsf(float2 a) { return std::hypot(a.x, a.y); }
