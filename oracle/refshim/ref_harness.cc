// Runs the reference's own CDI::phaseRetrieve (src/post_gpu/cdi.cc), built as
// host code from the reference sources, on a pattern and restart iterate from
// .bin files, and writes rho, Psi, the support field, the threshold and the
// residual.  Test infrastructure for the oracle pin.
//
// ref_harness <pattern.bin (centred float)> <restart.bin (complex, FFT order)>
//             <algorithm> <oversampling_spt> <shrinkThreshold> <exposure>
//             <simCCDbit> <noiseLevel> <out prefix> [prtfIter [saveState]]
// With prtfIter the reference also computes the PRTF from that iteration on
// and writes prtf.txt into the working directory (cdi.cc:355-380, 424-440);
// with saveState != 0 it then runs CDI::saveState (its plotted fields are
// dumped when CDXREF_PLOT_DUMP names a directory, its "mid=" line printed).
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "cdi.hpp"
#include "cudaConfig.hpp"
#include "imgio.hpp"

struct cudaVars {   // layout of __constant__ vars in src/gpu/cdi.cu:8-14
  int rcolor;
  Real beta_HIO;
  Real scale;
  Real threshold;
};
extern cudaVars vars;
extern "C" void writeFloatImage(const char* name, void* data, int row, int column);

// ref_harness --sim <intensity.bin> <phase.bin or -> <oversampling> <phaseModulation> <exposure> <out.bin>
//                   [<lambda> <pixelsize> <beamspotsize> <oversampling_spt> <isFresnel>]
// runs the noise-free simulation of readFiles/prepareIter (runSim, cdi.cc:62-82,
// 161-200) and writes the simulated patternData.  The optics set the distance as
// the constructor does for runSim (cdi.cc:39) and, with isFresnel, the Fresnel
// phase of the object (cdi.cc:174).
static int run_sim(int argc, char** argv) {
  if (argc < 8) return 2;
  CDI c("none.cfg");
  c.runSim = 1;
  c.common.Intensity = argv[2];
  c.common.Phase = strcmp(argv[3], "-") ? argv[3] : nullptr;
  c.oversampling = atof(argv[4]);
  c.phaseModulation = atof(argv[5]);
  c.exposure = atof(argv[6]);
  c.intensityModulation = 1;
  c.simCCDbit = 0;
  c.restart = 0;
  c.useBS = 0;
  c.verbose = 0;
  if (argc > 12) {
    c.lambda = atof(argv[8]);
    c.pixelsize = atof(argv[9]);
    c.beamspotsize = atof(argv[10]);
    c.oversampling_spt = atof(argv[11]);
    c.isFresnel = atoi(argv[12]);
    c.d = c.oversampling_spt * c.pixelsize * c.beamspotsize / c.lambda;
  }
  c.readFiles();
  c.init();
  c.prepareIter();
  writeFloatImage(argv[7], c.patternData, c.row, c.column);
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && !strcmp(argv[1], "--sim")) return run_sim(argc, argv);
  if (argc < 10) {
    fprintf(stderr, "usage: ref_harness pattern restart algorithm spt thr exposure ccd noise prefix\n");
    return 2;
  }
  CDI c("none.cfg");
  c.common.Pattern = argv[1];
  c.common.restart = argv[2];
  c.algorithm = argv[3];
  c.oversampling_spt = atof(argv[4]);
  c.shrinkThreshold = atof(argv[5]);
  c.exposure = atof(argv[6]);
  c.simCCDbit = atoi(argv[7]);
  c.noiseLevel = atoi(argv[8]);
  c.restart = 1;
  c.runSim = 0;
  c.useBS = 0;
  c.prtfIter = argc > 10 ? atoi(argv[10]) : 1 << 30;
  c.verbose = 0;
  c.readFiles();
  c.init();
  c.prepareIter();
  c.phaseRetrieve();
  const std::string pre = argv[9];
  if (argc > 11 && atoi(argv[11])) {
    writeComplexImage((pre + "_rho_before_save.bin").c_str(), c.objectWave, c.row, c.column);
    c.saveState();
    // checkAutoCorrelation (cdi.cc:231-239) takes rows*cols floats from the pool and has
    // the R2C write rows*(cols/2+1) complex into them, rows*8 bytes past the end; the
    // pool is handed a block of the half spectrum's size under that request's size
    {
      const size_t asked = (size_t)c.row * c.column * sizeof(Real);
      void* half = malloc((size_t)c.row * (c.column / 2 + 1) * sizeof(complexFormat));
      memMngr.registerMem(half, asked);
      memMngr.returnCache(half);
    }
    c.checkAutoCorrelation();   // util/cdi.cpp:47: plotted as "autocorrelation"
  }
  writeComplexImage((pre + "_rho.bin").c_str(), c.objectWave, c.row, c.column);
  writeComplexImage((pre + "_psi.bin").c_str(), c.patternWave, c.row, c.column);
  writeFloatImage((pre + "_support.bin").c_str(), c.support, c.row, c.column);
  FILE* f = fopen((pre + "_scalars.txt").c_str(), "w");
  fprintf(f, "threshold %.9g\nresidual %.9g\n", (double)vars.threshold, (double)c.residual);
  fclose(f);
  return 0;
}
