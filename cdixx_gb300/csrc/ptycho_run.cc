// ptycho_run <config>: the config-driven ptychography program, the counterpart
// of the reference's util/ptycho.cpp main() on this library.
//   runSim: object from InputImages.default.Intensity (and .Phase) .bin images,
//     pupil from InputImages.pupil.Intensity, probe = the pupil propagated by
//     dpupil, scan positions of initScan_triangle (written to scan.txt), and
//     noise-free patterns (createPattern) written as <Pattern><i>.bin, centred
//     and scaled by the exposure, as the reference saves them;
//   otherwise: patterns <outputDir><Pattern><i>.bin and positions from
//     <outputDir><distFile> (readPattern / readScan).
// Then initObject and, with doIteration, ptycho::iterate for nIter sweeps
// (scan orders: the rand() shuffle of a process that never seeded it); the
// object, the probe and the pupil are written to the output directory as
// ptycho_object.bin, ptycho_probe.bin, ptycho_pupil.bin.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "cdx_ptycho.h"
#include "readConfig.hpp"

namespace {

void die(const std::string& msg) {
  fprintf(stderr, "%s: %s\n", msg.c_str(), cdx_last_error());
  exit(1);
}

std::vector<float> read_image(const std::string& path, int& rows, int& cols) {
  int cplx = 0;
  if (cdx_read_bin(path.c_str(), &rows, &cols, &cplx, nullptr, 0) != CDX_OK) die("cannot read " + path);
  if (cplx) die(path + " must be a float image");
  std::vector<float> v((size_t)rows * cols);
  if (cdx_read_bin(path.c_str(), &rows, &cols, &cplx, v.data(), v.size()) != CDX_OK) die("cannot read " + path);
  return v;
}

// createWaveFront(intensity, phase, wave, 1) (src/gpu/cudaConfig.cu:710-732): sqrt(I) e^{i 2 pi (p - 0.5)}
std::vector<float> wavefront(const std::vector<float>& inten, const std::vector<float>* phase) {
  std::vector<float> w(2 * inten.size());
  for (size_t i = 0; i < inten.size(); ++i) {
    const float mod = std::sqrt(std::max(0.f, inten[i]));
    const float ph = phase ? (float)(((*phase)[i] - 0.5) * 2 * M_PI) : 0.f;
    w[2 * i] = mod * std::cos(ph);
    w[2 * i + 1] = mod * std::sin(ph);
  }
  return w;
}

// initScan_triangle (util/ptycho.cpp:139-175): 3 x 3 grid without (2, 1), odd
// columns shifted half a step and the middle one stretched, centred on the object
void scan_triangle(int row_O, int col_O, int row, int col, float step, float res, const std::string& out,
                   std::vector<float>& sx, std::vector<float>& sy) {
  std::ofstream f(out + "scan.txt");
  f << step * res << "\n";
  int maxx = 0, maxy = 0, minx = row_O, miny = row_O, i = 0;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      if (a == 2 && b == 1) continue;
      float xstep = (float)(a + (b % 2 == 0 ? 0 : 0.5));
      const float ystep = (float)b;
      if (b == 1) xstep = xstep * 2 - 1;
      f << i++ << " " << ystep << " " << xstep << "\n";
      sy.push_back(xstep * step);
      sx.push_back(ystep * step);
      maxx = std::max(maxx, (int)sx.back());
      maxy = std::max(maxy, (int)sy.back());
      minx = std::min(minx, (int)sx.back());
      miny = std::min(miny, (int)sy.back());
    }
  for (size_t k = 0; k < sx.size(); ++k) {
    sx[k] -= (minx + maxx - row_O + row) >> 1;
    sy[k] -= (miny + maxy - col_O + col) >> 1;
  }
}

// readScan (util/ptycho.cpp:88-123): first line the step in length units, then "i x y" in steps
int read_scan(const std::string& path, float res, std::vector<float>& sx, std::vector<float>& sy) {
  std::ifstream f(path);
  if (!f) die("cannot open " + path);
  std::string line;
  std::getline(f, line);
  const float step = (float)(std::atof(line.c_str()) / res);
  float maxxy = 0;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    int i;
    float x, y;
    if (!(is >> i >> x >> y)) continue;
    maxxy = std::max(maxxy, std::max(x, y));
    sx.push_back(x * step);
    sy.push_back(y * step);
  }
  return (int)(maxxy * step);
}

void shift_centre(std::vector<float>& a, int rows, int cols, bool to_centre) {   // cudaConvertFO, even sizes
  std::vector<float> b(a.size());
  for (int x = 0; x < rows; ++x)
    for (int y = 0; y < cols; ++y) {
      const int xs = (x + rows / 2) % rows, ys = (y + cols / 2) % cols;
      if (to_centre) b[(size_t)xs * cols + ys] = a[(size_t)x * cols + y];
      else b[(size_t)x * cols + y] = a[(size_t)xs * cols + ys];
    }
  a.swap(b);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    printf("usage: ptycho_run <config>\n");
    return 2;
  }
  readConfig cfg(argv[1]);
  const std::string out = cfg.outputDir ? cfg.outputDir : "./";
  cdx_pty_params p;
  cdx_pty_params_default(&p);
  p.lambda = cfg.lambda;
  p.d = cfg.d;
  p.dpupil = cfg.dpupil;
  p.pixelsize = cfg.pixelsize;
  p.pupil_size = cfg.pupilSize;
  p.exposure = cfg.exposure > 0 ? cfg.exposure : 1;
  p.mpie = cfg.mPIE;
  p.use_bs = cfg.useBS;
  p.beam_stop_size = cfg.beamStopSize;
  p.noise_level = cfg.noiseLevel;
  p.position_uncertainty = cfg.positionUncertainty;
  p.zernike_iter = cfg.zernikeIter;
  p.is_fresnel = cfg.isFresnel;
  std::vector<float> sx, sy, obj_truth, pupil, pats;
  if (cfg.runSim) {
    if (!cfg.common.Intensity || !cfg.pupil.Intensity) die("runSim needs InputImages.default.Intensity and .pupil.Intensity");
    int orow, ocol, prow, pcol;
    std::vector<float> inten = read_image(cfg.common.Intensity, orow, ocol), phase;
    if (cfg.common.Phase) {
      int r2, c2;
      phase = read_image(cfg.common.Phase, r2, c2);
      if (r2 != orow || c2 != ocol) die("the phase image must match the intensity image");
    }
    obj_truth = wavefront(inten, phase.empty() ? nullptr : &phase);
    pupil = wavefront(read_image(cfg.pupil.Intensity, prow, pcol), nullptr);
    p.obj_rows = orow;
    p.obj_cols = ocol;
    p.rows = prow;
    p.cols = pcol;
    const float res = (float)(cfg.lambda * cfg.d / cfg.pixelsize / prow);
    scan_triangle(orow, ocol, prow, pcol, (float)cfg.stepSize, res, out, sx, sy);
  } else {
    if (!cfg.common.Pattern) die("InputImages.default.Pattern is not set");
    int prow, pcol;
    std::vector<float> first = read_image(out + cfg.common.Pattern + "0.bin", prow, pcol);
    const float res = (float)(cfg.lambda * cfg.d / cfg.pixelsize / prow);
    const int maxxy = read_scan(out + cfg.distFile, res, sx, sy);
    p.rows = prow;
    p.cols = pcol;
    p.obj_rows = p.obj_cols = (int)(maxxy + prow + 3) / 4 * 4;
    const size_t n = (size_t)prow * pcol;
    pats.resize(n * sx.size());
    for (size_t i = 0; i < sx.size(); ++i) {
      int r, c;
      std::vector<float> im = i == 0 ? first : read_image(out + cfg.common.Pattern + std::to_string(i) + ".bin", r, c);
      shift_centre(im, prow, pcol, false);   // cudaConvertFO, then applyNorm(1/exposure)
      for (size_t k = 0; k < n; ++k) pats[i * n + k] = (float)(im[k] * (1. / p.exposure));
    }
  }
  p.nscan = (int)sx.size();
  const float resolution = (float)(cfg.lambda * cfg.d / cfg.pixelsize / p.rows);
  printf("Imaging distance = %4.2fcm\nResolution = %4.2fum\npupil - sample distance = %4.2fcm\n", cfg.d * 1e-4,
         resolution, cfg.dpupil * 1e-4);
  printf("Object image dimension (%d,%d)\nPupil image dimension (%d,%d)\n", p.obj_rows, p.obj_cols, p.rows, p.cols);
  cdx_pty* t = nullptr;
  if (cdx_pty_create(&p, nullptr, &t) != CDX_OK) die("cdx_pty_create");
  if (cdx_pty_set_scan(t, sx.data(), sy.data()) != CDX_OK) die("cdx_pty_set_scan");
  const size_t n = (size_t)p.rows * p.cols;
  if (cfg.runSim) {
    if (cdx_pty_set_object(t, obj_truth.data()) != CDX_OK || cdx_pty_set_pupil(t, pupil.data()) != CDX_OK ||
        (cfg.simCCDbit ? cdx_pty_simulate_ccd(t, 0x5eedull) : cdx_pty_simulate(t)) != CDX_OK)   // simCCDbit: ccdRecord
      die("createPattern");
    pats.resize(n * p.nscan);
    if (cdx_pty_get_patterns(t, pats.data()) != CDX_OK) die("cdx_pty_get_patterns");
    for (int i = 0; i < p.nscan; ++i) {   // saved centred and times the exposure
      std::vector<float> im(pats.begin() + i * n, pats.begin() + (i + 1) * n);
      for (float& v : im) v = (float)(v * p.exposure);
      shift_centre(im, p.rows, p.cols, true);
      const std::string name = out + (cfg.common.Pattern ? cfg.common.Pattern : "pattern") + std::to_string(i) + ".bin";
      cdx_write_bin(name.c_str(), im.data(), p.rows, p.cols, 0);
    }
  } else if (cdx_pty_set_patterns(t, pats.data()) != CDX_OK) {
    die("cdx_pty_set_patterns");
  }
  const unsigned long long seed = cfg.seed > 0 ? (unsigned long long)cfg.seed : 1ull;
  if (cdx_pty_init_object(t, seed) != CDX_OK) die("initObject");
  if (cfg.doIteration) {
    if (cdx_pty_iterate(t, 0, cfg.nIter, nullptr, 1) != CDX_OK) die("iterate");
    float ms = 0;
    cdx_pty_last_ms(t, &ms);
    printf("iterations: %d in %.3f ms\n", cfg.nIter, ms);
  }
  std::vector<float> obj((size_t)2 * p.obj_rows * p.obj_cols), pr(2 * n), pu(2 * n);
  if (cdx_pty_get_object(t, obj.data()) != CDX_OK || cdx_pty_get_probe(t, pr.data()) != CDX_OK ||
      cdx_pty_get_pupil(t, pu.data()) != CDX_OK)
    die("outputs");
  cdx_write_bin((out + "ptycho_object.bin").c_str(), obj.data(), p.obj_rows, p.obj_cols, 1);
  cdx_write_bin((out + "ptycho_probe.bin").c_str(), pr.data(), p.rows, p.cols, 1);
  cdx_write_bin((out + "ptycho_pupil.bin").c_str(), pu.data(), p.rows, p.cols, 1);
  cdx_pty_destroy(t);
  return 0;
}
