// The CDI class of the drop-in C++ layer (include/cdi.hpp), built on the C
// ABI.  Method by method it follows src/post_gpu/cdi.cc of the reference:
// the GPU work of each step is one cdx_* call, host-side file handling and
// error exits are kept as the reference has them.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cdi.hpp"

namespace {

std::vector<float> read_float_image(const char* path, int& rows, int& cols, bool& is_complex) {
  int z = 0;
  if (cdx_read_bin(path, &rows, &cols, &z, nullptr, 0) != CDX_OK) {
    fprintf(stderr, "ERROR: %s\n", cdx_last_error());
    exit(EXIT_FAILURE);
  }
  is_complex = z != 0;
  std::vector<float> v((size_t)rows * cols * (z ? 2 : 1));
  if (cdx_read_bin(path, &rows, &cols, &z, v.data(), v.size()) != CDX_OK) {
    fprintf(stderr, "ERROR: %s\n", cdx_last_error());
    exit(EXIT_FAILURE);
  }
  return v;
}

std::string out_path(const char* dir, const std::string& name) {
  std::string d = dir ? dir : "./";
  if (!d.empty() && d.back() != '/') d.push_back('/');
  return d + name;
}

}  // namespace

CDI::CDI(const char* configfile) : readConfig(configfile) {
  if (verbose >= 4) print();
  if (runSim) d = oversampling_spt * pixelsize * beamspotsize / lambda;   // cdi.cc:39
}

CDI::~CDI() {
  if (autoCorrelation) cudaFree(autoCorrelation);
  if (ctx_) cdx_destroy(ctx_);
}

void CDI::check(int code, const char* what) {
  if (code != CDX_OK) {
    fprintf(stderr, "%s: %s\n", what, cdx_last_error());
    exit(EXIT_FAILURE);
  }
}

void CDI::allocateMem() {   // cdi.cc:42-61
  if (ctx_) return;
  printf("allocating memory\n");
  cdx_params p;
  cdx_params_default(&p);
  p.rows = row;
  p.cols = column;
  p.batch = 1;
  p.beta = (float)beta;
  p.shrink_threshold = (float)shrinkThreshold;
  p.oversampling_spt = oversampling_spt > 0 ? (float)oversampling_spt : 2.f;
  p.exposure = exposure > 0 ? (float)exposure : 1.f;
  p.sim_ccd_bit = simCCDbit;
  p.noise_level = noiseLevel;
  p.shrink_mode = shrinkMode;
  p.sigma0 = (float)sigma0;
  p.sigma_min = (float)sigmaMin;
  p.sigma_decay = (float)sigmaDecay;
  p.prtf_iter = prtfIter;   // readConfig default 1000, as the reference
  check(cdx_create(&p, nullptr, &ctx_), "allocateMem");
  float* pd = nullptr;
  void* pw = nullptr;
  void* ow = nullptr;
  float* sp = nullptr;
  check(cdx_device_arrays(ctx_, &pd, &pw, &ow, &sp), "allocateMem");
  patternData = pd;
  patternWave = (complexFormat*)pw;
  objectWave = (complexFormat*)ow;
  support = sp;
}

// runSim (cdi.cc:62-82, 161-200): object from the Intensity (and Phase) .bin
// images, centred in a field `oversampling` times larger; the pattern is
// |FFT(object)|^2/N, optionally behind the beamstop.
void CDI::readObjectWave() {
  int r = 0, c = 0;
  bool z = false;
  if (!common.Intensity) {
    fprintf(stderr, "runSim needs InputImages.default.Intensity\n");
    exit(EXIT_FAILURE);
  }
  std::vector<float> inten = read_float_image(common.Intensity, r, c, z);
  std::vector<float> phase;
  if (phaseModulation && common.Phase) {
    int pr = 0, pc = 0;
    bool pz = false;
    phase = read_float_image(common.Phase, pr, pc, pz);
    if (pr != r || pc != c || pz) {
      fprintf(stderr, "Phase image must match the intensity image\n");
      exit(EXIT_FAILURE);
    }
  }
  const double os = oversampling > 0 ? oversampling : 1;
  row = (int)(r * os);
  column = (int)(c * os);
  allocateMem();
  // createWaveFront(intensity, phase, objectWave, objrow, objcol) (cudaConfig.cu:688-708)
  std::vector<float> obj((size_t)row * column * 2, 0.f);
  const int mx = (row - r) / 2, my = (column - c) / 2;
  for (int x = 0; x < r; ++x)
    for (int y = 0; y < c; ++y) {
      const float I = inten[(size_t)x * c + y];
      const float mod = intensityModulation ? std::sqrt(std::max(0.f, I)) : 1.f;
      float ph = 0.f;
      if (!phase.empty()) ph = (float)((phase[(size_t)x * c + y] * phaseModulation - 0.5) * 2 * M_PI);
      const size_t o = ((size_t)(x + mx) * column + (y + my)) * 2;
      obj[o] = mod * std::cos(ph);
      obj[o + 1] = mod * std::sin(ph);
    }
  // pattern = |FFT(obj)|^2 / N on the device (myFFT + convertFOPhase(1/sqrt N) + getMod2),
  // the object first multiplied by the Fresnel phase with isFresnel (cdi.cc:174)
  void* dev = nullptr;
  if (cudaMalloc(&dev, obj.size() * sizeof(float)) != cudaSuccess) check(CDX_ERR_NOMEM, "readObjectWave");
  cudaMemcpy(dev, obj.data(), obj.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (isFresnel)
    check(cdx_fresnel_phase(dev, row, column, 1, cdx_fresnel_factor(lambda, d, pixelsize, row, 0), nullptr),
          "readObjectWave");
  check(cdx_fft2(dev, dev, row, column, 1, 0, nullptr), "readObjectWave");
  cudaMemcpy(obj.data(), dev, obj.size() * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(dev);
  std::vector<float> pat((size_t)row * column);
  const double n = (double)row * column;
  for (size_t i = 0; i < pat.size(); ++i)
    pat[i] = (float)(((double)obj[2 * i] * obj[2 * i] + (double)obj[2 * i + 1] * obj[2 * i + 1]) / n);
  if (simCCDbit) {
    // detector quantisation and dark noise (applyPoissonNoise_WO, cdi.cc:191-193)
    void* dp = nullptr;
    if (cudaMalloc(&dp, pat.size() * sizeof(float)) != cudaSuccess) check(CDX_ERR_NOMEM, "readObjectWave");
    cudaMemcpy(dp, pat.data(), pat.size() * sizeof(float), cudaMemcpyHostToDevice);
    const float ex = exposure > 0 ? (float)exposure : 1.f;
    check(cdx_ccd_noise((float*)dp, (long long)pat.size(), (float)noiseLevel, ex, 65535 /* rcolor, format.hpp:20 */,
                        seed_, nullptr),
          "readObjectWave");
    cudaMemcpy(pat.data(), dp, pat.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dp);
  }
  check(cdx_set_pattern(ctx_, 0, pat.data(), CDX_HOST, CDX_FFT_ORDER, 1.f), "readObjectWave");
}

void CDI::readPattern() {   // cdi.cc:83-108
  int r = 0, c = 0;
  bool z = false;
  if (!common.Pattern) {
    fprintf(stderr, "InputImages.default.Pattern is not set\n");
    exit(EXIT_FAILURE);
  }
  std::vector<float> pattern = read_float_image(common.Pattern, r, c, z);
  if (z) {
    fprintf(stderr, "ERROR: the pattern must be a float image\n");
    exit(EXIT_FAILURE);
  }
  if (cropPattern) {   // centred crop (crop<Real> with midx = midy = 0, cudaConfig.cu:348-358)
    std::vector<float> cr((size_t)cropPattern * cropPattern);
    const int ox = (r - cropPattern) / 2, oy = (c - cropPattern) / 2;
    for (int x = 0; x < cropPattern; ++x)
      for (int y = 0; y < cropPattern; ++y) cr[(size_t)x * cropPattern + y] = pattern[(size_t)(x + ox) * c + y + oy];
    pattern.swap(cr);
    r = c = cropPattern;
  }
  row = r;
  column = c;
  allocateMem();
  float maxs = 0.f;
  bool nan = false;
  for (float v : pattern) {
    if (v != v) nan = true;
    else if (v > maxs) maxs = v;
  }
  if (maxs < 1e-7f || nan) {
    printf("max = %f\n", nan ? NAN : maxs);
    exit(0);
  }
  const float scale = (float)(1. / (exposure > 0 ? exposure : 1.));
  check(cdx_set_pattern(ctx_, 0, pattern.data(), CDX_HOST, CDX_CENTERED, scale), "readPattern");
  printf("Created pattern data\n");
}

void CDI::readFiles() {   // cdi.cc:109-117
  if (runSim) {
    printf("running simulation, reading input images\n");
    readObjectWave();
  } else {
    printf("running reconstruction, reading input pattern\n");
    readPattern();
  }
}

void CDI::setPattern_c(complexFormat* pattern) {   // cdi.cc:118-122, pattern: device, centred
  std::vector<float> h((size_t)row * column * 2);
  cudaMemcpy(h.data(), pattern, h.size() * sizeof(float), cudaMemcpyDeviceToHost);
  std::vector<float> m((size_t)row * column);
  for (size_t i = 0; i < m.size(); ++i) m[i] = h[2 * i] * h[2 * i] + h[2 * i + 1] * h[2 * i + 1];
  check(cdx_set_pattern(ctx_, 0, m.data(), CDX_HOST, CDX_CENTERED, 1.f), "setPattern_c");
  check(cdx_random_start(ctx_, seed_), "setPattern_c");
}

void CDI::setPattern(Real* pattern) {   // cdi.cc:124-128, pattern: device, centred
  check(cdx_set_pattern(ctx_, 0, pattern, CDX_DEVICE, CDX_CENTERED, 1.f), "setPattern");
  check(cdx_random_start(ctx_, seed_), "setPattern");
}

void CDI::init() {   // cdi.cc:129-159
  allocateMem();
  if (useBS) {
    std::vector<float> bs((size_t)row * column, 0.f);
    if (BSimage && BSimage[0] != '\0') {
      int r = 0, c = 0;
      bool z = false;
      std::vector<float> img = read_float_image(BSimage, r, c, z);
      if (r != row || c != column || z) {
        fprintf(stderr, "Beam stop mask (%d, %d) is not of the same size as diffraction pattern (%d, %d)!\n", r, c,
                row, column);
        abort();
      }
      for (size_t i = 0; i < bs.size(); ++i) bs[i] = 1.f - img[i];   // invert after cudaConvertFO
      check(cdx_set_beamstop(ctx_, 0, bs.data(), CDX_HOST, CDX_CENTERED), "init");
    } else {
      // createBeamStop: circle of radius beamStopSize around the zero frequency (misc.cc:191-195)
      for (int x = 0; x < row; ++x)
        for (int y = 0; y < column; ++y) {
          const int xs = x >= row / 2 ? x - row / 2 : x + row / 2;
          const int ys = y >= column / 2 ? y - column / 2 : y + column / 2;
          const float dx = (float)(xs - (row >> 1)), dy = (float)(ys - (column >> 1));
          bs[(size_t)x * column + y] = std::sqrt(dx * dx + dy * dy) < (float)beamStopSize ? 1.f : 0.f;
        }
      check(cdx_set_beamstop(ctx_, 0, bs.data(), CDX_HOST, CDX_FFT_ORDER), "init");
    }
  }
  createSupport();
  seed_ = seed ? (unsigned long long)seed
               : (unsigned long long)std::chrono::system_clock::now().time_since_epoch().count();
}

void CDI::prepareIter() {   // cdi.cc:160-230
  if (restart && common.restart) {
    int r = 0, c = 0, z = 0;
    if (cdx_read_bin(common.restart, &r, &c, &z, nullptr, 0) == CDX_OK && r == row && c == column && z) {
      std::vector<float> wf((size_t)r * c * 2);
      check(cdx_read_bin(common.restart, &r, &c, &z, wf.data(), wf.size()), "prepareIter");
      check(cdx_set_initial(ctx_, 0, wf.data(), CDX_HOST), "prepareIter");
      return;
    }
    printf("Restart file size mismatch: %d!=%d || %d!=%d\n", r, row, c, column);
    restart = 0;   // the reference then keeps a stale patternWave; here the random start follows
  }
  check(cdx_random_start(ctx_, seed_++), "prepareIter");
}

// cdi.cc:231-239: the forward transform of the pattern (R2C filled to the full
// Hermitian spectrum) times 1/sqrt(N), the buffer the reference plots, written as .bin
void CDI::checkAutoCorrelation() {
  const size_t n = (size_t)row * column;
  std::vector<float> pat(n), buf(2 * n, 0.f);
  cudaMemcpy(pat.data(), patternData, n * sizeof(float), cudaMemcpyDeviceToHost);
  for (size_t i = 0; i < n; ++i) buf[2 * i] = pat[i];
  if (!autoCorrelation && cudaMalloc((void**)&autoCorrelation, 2 * n * sizeof(float)) != cudaSuccess)
    check(CDX_ERR_NOMEM, "checkAutoCorrelation");
  cudaMemcpy(autoCorrelation, buf.data(), buf.size() * sizeof(float), cudaMemcpyHostToDevice);
  check(cdx_fft2(autoCorrelation, autoCorrelation, row, column, 1, 0, nullptr), "checkAutoCorrelation");
  cudaMemcpy(buf.data(), autoCorrelation, buf.size() * sizeof(float), cudaMemcpyDeviceToHost);
  const float s = (float)(1.0 / std::sqrt((double)n));
  for (float& v : buf) v *= s;
  cdx_write_bin(out_path(outputDir, "autocorrelation.bin").c_str(), buf.data(), row, column, 1);
}

void CDI::createSupport() {}   // the context builds the rect of oversampling_spt (cdi.cc:240-251)
void CDI::initSupport() {}     // reset by cdx_set_initial / cdx_random_start (cdi.cc:252-254)

complexFormat* CDI::phaseRetrieve() {   // cdi.cc:297-449
  const int e = cdx_run(ctx_, algorithm, &stats_);
  if (e == CDX_ERR_ALGO) {
    printf("%s\n", cdx_last_error());
    exit(0);
  }
  check(e, "phaseRetrieve");
  residual = (Real)stats_.residual;
  printf("residual= %f\n", residual);
  if (stats_.flags & 1) printf("max is ~0 or NaN at a shrinkwrap\n");
  // prtf.txt (cdi.cc:436-440) when the run reached prtfIter
  std::vector<float> prtf(row / 2);
  if (cdx_get_prtf(ctx_, 0, prtf.data(), CDX_HOST) == CDX_OK) {
    if (FILE* f = fopen("prtf.txt", "w")) {
      for (int i = 0; i < row / 2; ++i) fprintf(f, "%d, %f\n", i, prtf[i]);
      fclose(f);
    }
  }
  return patternWave;
}

void CDI::saveState() {   // cdi.cc:255-294: restart file of Psi plus .bin dumps of rho and the support
  const size_t n = (size_t)row * column;
  std::vector<float> psi(2 * n), rho(2 * n), spt(n);
  check(cdx_get_fourier(ctx_, 0, psi.data(), CDX_HOST), "saveState");
  check(cdx_get_object(ctx_, 0, rho.data(), CDX_HOST), "saveState");
  check(cdx_get_support(ctx_, 0, spt.data(), CDX_HOST), "saveState");
  if (common.restart) cdx_write_bin(common.restart, psi.data(), row, column, 1);
  cdx_write_bin(out_path(outputDir, "recon_object" + save_suffix + ".bin").c_str(), rho.data(), row, column, 1);
  for (float& v : spt) v = v > stats_.threshold ? 1.f : 0.f;   // bitMap(support, support)
  cdx_write_bin(out_path(outputDir, "support" + save_suffix + ".bin").c_str(), spt.data(), row, column, 0);
  if (isFresnel) {   // cdi.cc:285-288: the object's phase with the Fresnel phase removed
    std::vector<float> rf(rho);
    void* dev = nullptr;
    if (cudaMalloc(&dev, rf.size() * sizeof(float)) != cudaSuccess) check(CDX_ERR_NOMEM, "saveState");
    cudaMemcpy(dev, rf.data(), rf.size() * sizeof(float), cudaMemcpyHostToDevice);
    check(cdx_fresnel_phase(dev, row, column, 1, cdx_fresnel_factor(lambda, d, pixelsize, row, 1), nullptr),
          "saveState");
    cudaMemcpy(rf.data(), dev, rf.size() * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dev);
    std::vector<float> ph(n);
    for (size_t i = 0; i < n; ++i) ph[i] = std::atan2(rf[2 * i + 1], rf[2 * i]);
    cdx_write_bin(out_path(outputDir, "recon_phase_fresnelRemoved" + save_suffix + ".bin").c_str(), ph.data(), row,
                  column, 0);
  }

  // findMiddle (misc.cc:27-42): centroid of the support bitmap in units of the
  // field, coordinates (x + 0.5)/row - 0.5 (multiplyx/multiplyy, cudaConfig.cu:1427-1437)
  double s0 = 0, sx = 0, sy = 0;
  for (int x = 0; x < row; ++x)
    for (int y = 0; y < column; ++y) {
      const double m = spt[(size_t)x * column + y];
      s0 += m;
      sx += m * (float)((x + 0.5f) / row - 0.5f);
      sy += m * (float)((y + 0.5f) / column - 0.5f);
    }
  const float midx = s0 > 0 ? (float)(sx / s0) : 0.f, midy = s0 > 0 ? (float)(sy / s0) : 0.f;
  printf("mid= %f,%f\n", midx, midy);
  // crop (cudaConfig.cu:348-358) of the object to the support size around the centroid
  const double os = oversampling_spt > 0 ? oversampling_spt : 2.;
  const int row_spt = (int)(row / os), col_spt = (int)(column / os);
  int shiftx = (int)(row * midx);
  if (shiftx + row_spt / 2 > row / 2) shiftx = (row - row_spt) / 2;
  else if (shiftx - row_spt / 2 < -row / 2) shiftx = (row_spt - row) / 2;
  int shifty = (int)(column * midy);
  if (shifty + col_spt / 2 > column / 2) shifty = (row - col_spt) / 2;   // row, as the reference has it
  else if (shifty - col_spt / 2 < -column / 2) shifty = (col_spt - column) / 2;
  std::vector<float> crop((size_t)row_spt * col_spt * 2);
  for (int x = 0; x < row_spt; ++x)
    for (int y = 0; y < col_spt; ++y) {
      const long long t = (long long)(x + (row - row_spt) / 2 + shiftx) * column + y + (column - col_spt) / 2 + shifty;
      const size_t o = ((size_t)x * col_spt + y) * 2;
      if (t >= 0 && t < (long long)n) {
        crop[o] = rho[2 * t];
        crop[o + 1] = rho[2 * t + 1];
      }
    }
  cdx_write_bin(out_path(outputDir, "recon_wave" + save_suffix + ".bin").c_str(), crop.data(), row_spt, col_spt, 1);
  // autocorrelation of the reconstruction: FFT(|Psi|^2) (cdi.cc:289-292)
  std::vector<float> ac(2 * n, 0.f);
  for (size_t i = 0; i < n; ++i) ac[2 * i] = psi[2 * i] * psi[2 * i] + psi[2 * i + 1] * psi[2 * i + 1];
  void* d = nullptr;
  if (cudaMalloc(&d, ac.size() * sizeof(float)) != cudaSuccess) check(CDX_ERR_NOMEM, "saveState");
  cudaMemcpy(d, ac.data(), ac.size() * sizeof(float), cudaMemcpyHostToDevice);
  check(cdx_fft2(d, d, row, column, 1, 0, nullptr), "saveState");
  cudaMemcpy(ac.data(), d, ac.size() * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  cdx_write_bin(out_path(outputDir, "autocorrelation_recon.bin").c_str(), ac.data(), row, column, 1);
}
