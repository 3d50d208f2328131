// Definitions the reference's ptychography driver (util/ptycho.cpp) links
// against but never reaches with the settings the pin uses.  Test
// infrastructure for the oracle pin.
#include <cstdlib>

#include "cdxref_defs.h"
#include "format.hpp"

char shared_mem[1];   // the extern __shared__ buffer of phaseUnwrapping (never launched here)
// the extern __shared__ buffer of the Zernike/Laguerre projections
// (src/gpu/beamDecomposition.cu): one block runs at a time under cdxref::coop
alignas(16) char shared_raw[1 << 16];
