// Replacement for the reference's kernel-definition macros (include/cudaDefs_h.cu)
// under host emulation: same macro names and argument conventions, but each
// "launch" runs the kernel body once per emulated thread.  Defining the
// header guard keeps the reference's own version out.
#pragma once
#define __CUDADEFS_H__
#include "cdxref_host.h"
#include "cuda_runtime.h"
#include "cuComplex.h"
#include "format.hpp"
#define cuComplex float2
#define crealf(z) (__real__(z))
#define cimagf(z) (__imag__(z))
#define addVar(args...) cuda_imgsz.x, cuda_imgsz.y, args
#define addVarArg(x...) int cuda_row, int cuda_column, x
#define addVar3D(args...) cuda_imgsz.x, cuda_imgsz.y, cuda_imgsz.z, args
#define addVarArg3D(x...) int cuda_row, int cuda_column, int cuda_height, x
#define CDXREF_RUN(grid, block, call) for (cdxref::Launch cdxref_l_(grid, block); cdxref_l_.next();) call
#define cuFunc(name, args, param, content...) \
  void name##Wrap(addVarArg args) content     \
  void name args { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap(addVar param)); }
#define cuFunc3D(name, args, param, content...) \
  void name##Wrap(addVarArg3D args) content     \
  void name args { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap(addVar3D param)); }
#define cuFuncc(name, argsf, argsw, param, content...) \
  void name##Wrap(addVarArg argsw) content             \
  void name argsf { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap(addVar param)); }
#define cuFuncc3D(name, argsf, argsw, param, content...) \
  void name##Wrap(addVarArg3D argsw) content             \
  void name argsf { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap(addVar3D param)); }
#define cuFuncTemplate(name, args, param, content...) \
  template <typename T>                               \
  void name##Wrap(addVarArg args) content             \
  template <typename T>                               \
  void name args { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap<T>(addVar param)); }
#define cuFunccTemplate(name, argsf, argsw, param, content...) \
  template <typename T>                                        \
  void name##Wrap(addVarArg argsw) content                     \
  template <typename T>                                        \
  void name argsf { CDXREF_RUN(numBlocks, threadsPerBlock, name##Wrap(addVar param)); }
#define addSize(args...) size_t size, args
#define cuFuncSharedDec(funcname, ...) void funcname(size_t size, __VA_ARGS__)
#define cuFuncShared(name, args, param, content...)                                               \
  void name##Wrap(addVarArg args) content                                                         \
  void name(addSize args) {                                                                       \
    dim3 nthd(16, 16);                                                                            \
    dim3 nblk((cuda_imgsz.x - 1) / nthd.x + 1, (cuda_imgsz.y - 1) / nthd.y + 1);                  \
    CDXREF_RUN(nblk, nthd, name##Wrap(addVar param));                                             \
  }
#define cuda1Idx()                                   \
  int index = blockIdx.x * blockDim.x + threadIdx.x; \
  if (index >= cuda_row * cuda_column) return;
#define cuda1Idx3D()                                 \
  int index = blockIdx.x * blockDim.x + threadIdx.x; \
  if (index >= cuda_row * cuda_column * cuda_height) return;
#define cudaIdx()                                    \
  int index = blockIdx.x * blockDim.x + threadIdx.x; \
  if (index >= cuda_row * cuda_column) return;       \
  int x = index / cuda_column;                       \
  int y = index % cuda_column;
#define cuda3Idx()                                                \
  int index = blockIdx.x * blockDim.x + threadIdx.x;              \
  if (index >= cuda_row * cuda_column * cuda_height) return;      \
  int z = index / (cuda_row * cuda_column);                       \
  int idxxy = index - z * (cuda_row * cuda_column);               \
  int x = idxxy % cuda_row;                                       \
  int y = idxxy / cuda_row;
extern const dim3 threadsPerBlock;
extern dim3 numBlocks;
extern dim3 cuda_imgsz;
