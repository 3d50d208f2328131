// Definitions the reference's hot-path sources need from subsystems outside
// the CDI iteration (plotting, image codecs, MNIST, Fresnel propagation,
// FISTA), as no-ops or minimal .bin restatements, plus the host-emulation
// globals.  Test infrastructure for the oracle pin only.
#include <map>
#include <string>
#include <cstdlib>

#include "cdxref_defs.h"
#include "cufft.h"
#include "cuPlotter.hpp"
#include "imgio.hpp"
#include "memManager.hpp"
#include "misc.hpp"
#include "mnistData.hpp"
#include "propagator.hpp"
#include "tvFilter.hpp"

thread_local uint3_t blockIdx, threadIdx;
thread_local dim3 blockDim, gridDim;
thread_local cdxref::BlockBarrier* cdxref::tl_block_barrier = nullptr;
std::map<int, cdxref_plan>& cdxref_plans() { static std::map<int, cdxref_plan> m; return m; }
float tile[1];   // the extern __shared__ tile of applyConvolution (never launched here)

// The plotter draws nothing.  With CDXREF_PLOT_DUMP set to a directory, every
// plotted field is written there raw as <label>.bin (the array the reference
// hands to the plotter, at the size of the last init), so the harness can
// record what saveState computes (cdi.cc:255-294).
extern "C" void writeComplexImage(const char* name, void* data, int row, int column);
extern "C" void writeFloatImage(const char* name, void* data, int row, int column);
static int cdxref_plt_rows = 0, cdxref_plt_cols = 0;
static void cdxref_plot_dump(const char* label, void* data, bool cplx) {
  const char* dir = getenv("CDXREF_PLOT_DUMP");
  if (!dir || !data || !label || cdxref_plt_rows <= 0 || cdxref_plt_cols <= 0) return;
  const std::string path = std::string(dir) + "/" + label + ".bin";
  if (cplx) writeComplexImage(path.c_str(), data, cdxref_plt_rows, cdxref_plt_cols);
  else writeFloatImage(path.c_str(), data, cdxref_plt_rows, cdxref_plt_cols);
}
cuPlotter plt;
void cuPlotter::init(int r, int c, const char*) { cdxref_plt_rows = r; cdxref_plt_cols = c; }
int cuPlotter::initVideo(const char*, int, bool, bool) { return 0; }
void cuPlotter::saveVideo(int) {}
void cuPlotter::saveFloat(void*, const char*) {}
void cuPlotter::saveComplex(void*, const char*) {}
void cuPlotter::plotComplex(void* d, const mode, bool, Real, const char* label, bool, bool, bool, const char*) {
  cdxref_plot_dump(label, d, true);
}
void cuPlotter::plotComplexColor(void* d, bool, Real, const char* label, bool, bool) { cdxref_plot_dump(label, d, true); }
void cuPlotter::plotFloat(void* d, const mode, bool, Real, const char* label, bool, bool, bool, const char*) {
  cdxref_plot_dump(label, d, false);
}
cuPlotter::~cuPlotter() {}

// .bin images: 20-byte header {char type; int rows, cols, nchann, typesize}, then data
Real* readImage(const char* name, int& row, int& col, void* (*)(size_t)) {
  FILE* f = fopen(name, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", name); abort(); }
  imageFile h;
  if (fread(&h, sizeof h, 1, f) != 1 || (h.type != FLOAT && h.type != FLOAT2)) abort();
  row = h.rows;
  col = h.cols;
  size_t n = (size_t)row * col * (h.type == FLOAT2 ? 2 : 1);
  Real* p = (Real*)ccmemMngr.borrowCache(n * sizeof(Real));   // released by returnCache (cdi.cc:103)
  if (fread(p, sizeof(Real), n, f) != n) abort();
  fclose(f);
  return p;
}
extern "C" void writeComplexImage(const char* name, void* data, int row, int column) {
  FILE* f = fopen(name, "wb");
  imageFile h;
  memset(&h, 0, sizeof h);
  h.type = FLOAT2;
  h.rows = row;
  h.cols = column;
  fwrite(&h, sizeof h, 1, f);
  fwrite(data, sizeof(Real) * 2, (size_t)row * column, f);
  fclose(f);
}
extern "C" void writeFloatImage(const char* name, void* data, int row, int column) {
  FILE* f = fopen(name, "wb");
  imageFile h;
  memset(&h, 0, sizeof h);
  h.type = FLOAT;
  h.rows = row;
  h.cols = column;
  fwrite(&h, sizeof h, 1, f);
  fwrite(data, sizeof(Real), (size_t)row * column, f);
  fclose(f);
}
#ifndef CDXREF_WITH_MISC
complexFormat findMiddle(Real*, int) { return 0; }
complexFormat findMiddle(complexFormat*, int) { return 0; }
Real* createBeamStop(int, int, int) { abort(); }
void readComplexWaveFront(const char*, const char*, Real*&, Real*&, int&, int&) { abort(); }
#endif
#ifndef CDXREF_WITH_FISTA
void FISTA(Real*, Real*, Real, int, void (*)(Real*, Real*)) { abort(); }
#endif
mnistData::mnistData(const char*) {}
mnistData::~mnistData() {}
cuMnist::cuMnist(const char* d, int, int, int, int) : mnistData(d) {}
void cuMnist::cuRead(void*) { abort(); }
#ifndef CDXREF_WITH_PTYCHO_KERNELS
// phase unwrapping of src/post_gpu/misc.cc calls two kernels of src/gpu/ptycho.cu
void phaseUnwrapping(Real*) { abort(); }
void solve_poisson_frequency_domain(complexFormat*) { abort(); }
#endif
#ifndef CDXREF_WITH_PROPAGATOR
void propagator::multiplyFresnelPhase(complexFormat*) { abort(); }
void propagator::removeFresnelPhase(complexFormat*) { abort(); }
#endif
