// Runs the reference's own ptychographic reconstruction, ptycho::iterate
// (util/ptycho.cpp:429-736, with the kernels of src/gpu/ptycho.cu and
// src/gpu/cudaConfig.cu), built as host code from the reference sources, on
// an object, a probe, diffraction patterns and scan positions read from
// files, and writes the reconstructed object and pupil.  The reference's
// driver file is compiled into this translation unit (its path comes from
// the build recipe as CDXREF_PTYCHO_CPP; its main() is renamed).
// Test infrastructure for the oracle pin.
//
// pty_harness <object.bin> <probe.bin> <patterns.bin (nscan stacked, FFT order,
//             scaled 1/exposure)> <scan.txt ("x y" per line)> <nIter> <mPIE>
//             <lambda> <d> <dpupil> <pixelsize> <pupilSize> <exposure>
//             <useBS> <beamStopSize> <rand seed> <out prefix>
//             [noiseLevel [zernikeIter [isFresnel [positionUncertainty]]]]
// (zernikeIter > 0 runs the FISTA object step, the probe momentum and, from
// iteration 400, the Zernike pupil fit; isFresnel the exit wave's Fresnel phase;
// positionUncertainty > 0 the scan-position refinement every 20 sweeps from 500)
#define main cdxref_ptycho_main
#include CDXREF_PTYCHO_CPP
#undef main

#include <cstdlib>
#include <fstream>
#include <vector>

extern "C" void writeComplexImage(const char* name, void* data, int row, int column);

static std::vector<float> cdxref_read_bin(const char* name, int& rows, int& cols, int& comps) {
  FILE* f = fopen(name, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", name); exit(2); }
  imageFile h;
  if (fread(&h, sizeof h, 1, f) != 1) exit(2);
  rows = h.rows;
  cols = h.cols;
  comps = h.type == FLOAT2 ? 2 : 1;
  fseek(f, 0, SEEK_END);
  const long bytes = ftell(f) - (long)sizeof h;
  fseek(f, sizeof h, SEEK_SET);
  std::vector<float> v(bytes / sizeof(float));
  if (fread(v.data(), sizeof(float), v.size(), f) != v.size()) exit(2);
  fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 17) {
    fprintf(stderr, "usage: pty_harness object probe patterns scan nIter mPIE lambda d dpupil pixelsize "
                    "pupilSize exposure useBS beamStopSize seed prefix\n");
    return 2;
  }
  ptycho p("none.cfg");
  p.verbose = 0;
  p.runSim = 0;
  p.isFresnel = argc > 19 ? atoi(argv[19]) : 0;
  p.saveVideoEveryIter = 0;
  p.computeErrorEveryIter = 0;
  p.zernikeIter = argc > 18 ? atoi(argv[18]) : 0;
  p.positionUncertainty = argc > 20 ? atof(argv[20]) : 0;
  p.nIter = atoi(argv[5]);
  p.mPIE = atoi(argv[6]);
  p.lambda = atof(argv[7]);
  p.d = atof(argv[8]);
  p.dpupil = atof(argv[9]);
  p.pixelsize = atof(argv[10]);
  p.pupilSize = atof(argv[11]);
  p.exposure = atof(argv[12]);
  p.useBS = atoi(argv[13]);
  p.beamStopSize = atoi(argv[14]);
  p.noiseLevel = argc > 17 ? atoi(argv[17]) : 0;
  // what the constructor would have taken from the config file
  p.propagate_esw.lambda = p.propagate_pupil.lambda = p.lambda;
  p.propagate_esw.distance = p.d;
  p.propagate_esw.pixelsize = p.pixelsize;
  p.propagate_pupil.distance = p.dpupil;

  int orow, ocol, oc, prow, pcol, pc, trow, tcol, tc;
  std::vector<float> obj = cdxref_read_bin(argv[1], orow, ocol, oc);
  std::vector<float> probe = cdxref_read_bin(argv[2], prow, pcol, pc);
  std::vector<float> pats = cdxref_read_bin(argv[3], trow, tcol, tc);
  if (oc != 2 || pc != 2 || tc != 1) { fprintf(stderr, "object/probe complex, patterns real\n"); return 2; }
  p.row = prow;
  p.column = pcol;
  p.row_O = orow;
  p.column_O = ocol;
  p.sz = prow * pcol * sizeof(Real);
  p.resolution = p.lambda * p.d / p.pixelsize / p.row;   // readPupilAndObject, util/ptycho.cpp:246

  std::vector<float> sx, sy;
  {
    std::ifstream f(argv[4]);
    float x, y;
    while (f >> x >> y) { sx.push_back(x); sy.push_back(y); }
  }
  p.nscan = (int)sx.size();
  p.allocScan();
  for (int i = 0; i < p.nscan; i++) { p.scanposx[i] = sx[i]; p.scanposy[i] = sy[i]; }
  p.allocateMem();
  memcpy(p.objectWave, obj.data(), sizeof(float) * 2 * orow * ocol);
  memcpy(p.pupilpatternWave, probe.data(), sizeof(float) * 2 * prow * pcol);
  const size_t npx = (size_t)prow * pcol;
  if (pats.size() != npx * p.nscan) { fprintf(stderr, "pattern stack size mismatch\n"); return 2; }
  for (int i = 0; i < p.nscan; i++) {
    p.patterns[i] = (Real*)memMngr.borrowCache(p.sz);
    memcpy(p.patterns[i], pats.data() + npx * i, p.sz);
  }
  resize_cuda_image(p.row, p.column);
  init_fft(p.row, p.column);   // as readPupilAndObject / readPattern do (util/ptycho.cpp:285, 710)
  if (p.useBS) p.beamstop = createBeamStop(p.row, p.column, p.beamStopSize);
  srand((unsigned)atoi(argv[15]));
  p.iterate();
  const std::string pre = argv[16];
  writeComplexImage((pre + "_object.bin").c_str(), p.objectWave, p.row_O, p.column_O);
  writeComplexImage((pre + "_pupil.bin").c_str(), p.pupilpatternWave, p.row, p.column);
  return 0;
}
