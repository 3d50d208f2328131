// Definitions the reference's ptychography driver (util/ptycho.cpp) links
// against but never reaches with the settings the pin uses (no Zernike pupil
// fit): aborting stubs.  Test infrastructure for the oracle pin.
#include <cstdlib>

#include "cdxref_defs.h"
#include "format.hpp"

char shared_mem[1];   // the extern __shared__ buffer of phaseUnwrapping (never launched here)
void* zernike_init(int, int, int) { return nullptr; }
void zernike_compute(void*, complexFormat*, Real, Real, Real) { abort(); }
void zernike_reconstruct(void*, complexFormat*, Real) { abort(); }
