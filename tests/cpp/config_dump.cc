// Prints the fields readConfig parsed from a config file and the step count
// and first steps of its algorithm, for tests/test_cpp_layer.py.
#include <cstdio>

#include "readConfig.hpp"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  readConfig c(argv[1]);
  printf("Pattern=%s\nrestart=%s\nIntensity=%s\npupilPattern=%s\n", c.common.Pattern ? c.common.Pattern : "",
         c.common.restart ? c.common.restart : "", c.common.Intensity ? c.common.Intensity : "",
         c.pupil.Pattern ? c.pupil.Pattern : "");
  printf("algorithm=%s\n", c.algorithm);
  printf("oversampling=%g\noversampling_spt=%g\nshrinkThreshold=%g\nexposure=%g\nlambda=%g\nd=%g\n", c.oversampling,
         c.oversampling_spt, c.shrinkThreshold, c.exposure, c.lambda, c.d);
  printf("beamStopSize=%d\nnIter=%d\nprtfIter=%d\nnoiseLevel=%d\nverbose=%d\n", c.beamStopSize, c.nIter, c.prtfIter,
         c.noiseLevel, c.verbose);
  printf("simCCDbit=%d\nuseBS=%d\ndoIteration=%d\nrestartFlag=%d\nrunSim=%d\nintensityModulation=%d\n", c.simCCDbit,
         c.useBS, c.doIteration, c.restart, c.runSim, c.intensityModulation);
  printf("beta=%g\nphotoncount=%g\nstepSize=%g\nBSimage=%s\n", c.beta, c.photoncount, c.stepSize, c.BSimage);
  AlgoParser a(c.algorithm);
  int n = 0, first[8];
  for (int s; (s = a.next()) >= 0; ++n)
    if (n < 8) first[n] = s;
  printf("steps=%d\nfirst=", n);
  for (int i = 0; i < n && i < 8; ++i) printf("%d,", first[i]);
  printf("\n");
  return 0;
}
