/* readConfig.hpp -- configuration of the GB300 CDI path, source-compatible
 * with the reference's include/readConfig.hpp (keys, types and defaults of
 * the `Job` group and the InputImages.default / InputImages.pupil files, and
 * the AlgoParser interface).  Config files use the libconfig syntax the
 * reference reads (html/default/cdi.cfg); this parser handles the subset
 * those files use: groups, scalar settings, strings, comments.
 */
#ifndef CDX_READCONFIG_HPP
#define CDX_READCONFIG_HPP

#include <memory>
#include <string>
#include <vector>

#define CDX_EXPORT __attribute__((visibility("default")))

struct CDIfiles {
  const char* Pattern = nullptr;
  const char* Intensity = nullptr;
  const char* Phase = nullptr;
  const char* restart = nullptr;
};

class CDX_EXPORT readConfig {
 public:
  // ---- int fields (reference readConfig.hpp:25-26)
  int beamStopSize = 5, nIter = 1, nIterpupil = 1, noiseLevel = 0, noiseLevel_pupil = 0, verbose = 2, mnistN = 3,
      cropPattern = 0, spectrumSamplingStep = 10, saveVideoEveryIter = 0, prtfIter = 1000, zernikeIter = 0,
      scanx = 3, scany = 3, computeErrorEveryIter = 0;
  // ---- bool fields (reference readConfig.hpp:28-29)
  bool isFlip = 0, runSim = 0, simCCDbit = 0, isFresnel = 0, doIteration = 0, useGaussionLumination = 0,
       useGaussionHERALDO = 0, doCentral = 0, useRectHERALDO = 0, dopupil = 0, useDM = 0, useBS = 0, reconAC = 0,
       phaseModulation_pupil = 0, intensityModulation = 1, restart = 0, saveIter = 0, domnist = 0, saveLMDB = 0,
       solveSpectrum = 0, mPIE = 1, online = 0;
  // ---- float fields (double, reference readConfig.hpp:31-32)
  double exposure = 0, exposurepupil = 0, oversampling = 0, oversampling_spt = 0, lambda = 0, d = 0, dpupil = 0,
         pixelsize = 0, beamspotsize = 0, shrinkThreshold = 0, positionUncertainty = 0, costheta = 1,
         photoncount = 1e9, phaseModulation = 0, stepSize = 64, pupilSize = 500;
  // ---- string fields (reference readConfig.hpp:34-35)
  const char* mnistData = "data";
  const char* algorithm = "1000*HIO";
  const char* ccd_response = "/home/boyang/SharedNTFS/images/ccd_response.txt";
  const char* spectrum = "/home/boyang/SharedNTFS/images/spectrum/spectrum_after_sample.txt";
  const char* BSimage = "";
  const char* outputDir = "./";
  const char* distFile = "./scan.txt";
  // ---- GB300 path settings (not in the reference; all optional in `Job`)
  double beta = 1.0;          // vars.beta_HIO of the real-space updates (the reference fixes it at 1)
  int shrinkMode = 0;         // 0: Fourier-domain Gaussian (CDI::phaseRetrieve), 1: |rho|^2 blur (holo)
  double sigma0 = 3, sigmaMin = 2, sigmaDecay = 0.99;
  long long seed = 0;         // random-phase start; 0: wall clock like the reference

  CDIfiles pupil;
  CDIfiles common;
  readConfig(const char* configfile);
  void print();
  ~readConfig() {}

 private:
  std::vector<std::unique_ptr<std::string>> strings_;   // storage of the string values
};

/* The algorithm-string parser (reference readConfig.hpp:37-48 /
 * readConfig.cc:82-163): next() returns the Algorithm code of each step in
 * order, -1 at the end; restart() rewinds. */
class CDX_EXPORT AlgoParser {
 public:
  AlgoParser(const char* formula);
  void restart();
  int next();
  int size() const { return (int)steps_.size(); }

 private:
  std::vector<int> steps_;
  size_t pos_ = 0;
};

#endif
