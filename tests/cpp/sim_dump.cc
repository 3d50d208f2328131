// Runs the runSim set-up of the C++ CDI layer (readFiles, init, prepareIter)
// on a config and writes the simulated pattern (patternData, a device array)
// to a .bin file, for tests/test_golden.py.
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "cdi.hpp"
#include "cdx.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  CDI c(argv[1]);
  c.readFiles();
  c.init();
  c.prepareIter();
  std::vector<float> h((size_t)c.row * c.column);
  if (cudaMemcpy(h.data(), c.patternData, h.size() * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
  return cdx_write_bin(argv[2], h.data(), c.row, c.column, 0) == CDX_OK ? 0 : 4;
}
