/* cdi.hpp -- the CDI class of the GB300 path, source-compatible with the
 * reference's include/cdi.hpp: same public fields and methods, so a driver
 * written against the reference (util/cdi.cpp: construct from a config file,
 * readFiles, init, prepareIter, phaseRetrieve, saveState) builds unchanged.
 *
 * patternData, patternWave, objectWave and support are DEVICE pointers into
 * the arena of the underlying cdx context (include/cdx.h), as in the
 * reference, and stay valid for the object's lifetime.  Image input/output is
 * the reference's .bin format; PNG/TIFF plotting is replaced by .bin dumps
 * under outputDir.  Errors print a message and exit like the reference
 * (cdi.cc:97-101, readConfig.cc:132-135).
 */
#ifndef CDX_CDI_HPP
#define CDX_CDI_HPP

#include <string>

#include "cdx.h"
#include "readConfig.hpp"

#ifndef Real
#define Real float
#endif
#ifndef complexFormat
#define complexFormat _Complex Real
#endif

enum Algorithm { RAAR, ER, POSER, HIO, POSHIO, FHIO, shrinkWrap, XCORRELATION, KKT, TV, cnt };

class CDX_EXPORT CDI : public readConfig {
 public:
  CDI(const char* configfile);
  ~CDI();
  Real* patternData = 0;
  Real* beamstop = 0;
  complexFormat* patternWave = 0;
  complexFormat* autoCorrelation = 0;
  int row = 0, column = 0;
  complexFormat* objectWave = 0;
  Real* support = 0;
  Real residual = 0;
  Real resolution = 0;
  void* cuda_spt = 0;
  void* mnist_dat = 0;
  std::string save_suffix = "";
  void* devstates = 0;
  void allocateMem();
  void readObjectWave();
  void readPattern();
  void readFiles();
  void setPattern(Real* pattern);
  void setPattern_c(complexFormat* pattern);
  void init();
  void prepareIter();
  void checkAutoCorrelation();
  void createSupport();
  void initSupport();
  complexFormat* phaseRetrieve();
  void saveState();

  // GB300 additions
  cdx_ctx* context() const { return ctx_; }
  const cdx_stats& lastStats() const { return stats_; }

 private:
  cdx_ctx* ctx_ = nullptr;
  cdx_stats stats_{};
  unsigned long long seed_ = 0;
  void check(int code, const char* what);
};

#endif
