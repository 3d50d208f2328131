// cdi_run <config>: the config-driven entry point, step for step the
// reference's util/cdi.cpp (construct CDI from the config, readFiles, init,
// prepareIter, phaseRetrieve + saveState, nIter restarts keeping the lowest
// residual, checkAutoCorrelation), on the GB300 path.
#include <cmath>
#include <cstdio>

#include "../../include/cdi.hpp"

int main(int argc, char** argv) {
  if (argc < 2) {
    printf("usage: cdi_run <config file>\n");
    return 1;
  }
  CDI setups(argv[1]);
  setups.readFiles();
  setups.init();
  printf("Imaging distance = %4.2fcm\n", setups.d * 1e-4);
  printf("pupil Imaging distance = %4.2fcm\n", setups.dpupil * 1e-4);
  const double fresnel = M_PI * setups.beamspotsize * setups.beamspotsize / (setups.d * setups.lambda);
  printf("Fresnel Number = %f\n", fresnel);
  // The reference's MNIST simulation loop (runSim with domnist) needs its MNIST
  // reader, which this build does not carry: the run goes on as a single pattern.
  if (setups.runSim && setups.domnist) printf("domnist: MNIST simulation not built, running one pattern\n");
  setups.prepareIter();
  if (setups.doIteration) {
    setups.phaseRetrieve();
    setups.saveState();
  }
  double smallresidual = setups.residual;
  for (int i = 0; i < setups.nIter; i++) {
    setups.prepareIter();
    if (setups.doIteration) {
      setups.phaseRetrieve();
      if (smallresidual > setups.residual) {
        smallresidual = setups.residual;
        setups.saveState();
      }
    }
  }
  setups.checkAutoCorrelation();
  return 0;
}
