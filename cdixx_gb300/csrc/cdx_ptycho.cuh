// Per-scan-position kernels of the ptychographic sweep, on the register-handoff
// FFT engine of cdx_rfft.cuh.  One position of ptycho::iterate
// (util/ptycho.cpp:514-560) is three launches:
//   forward row pass   psi = P * O_window, row FFT            -> W (column-tiled)
//   column pass        column FFT, applyModAccurate, column IFFT -> W
//   update row pass    row IFFT * norm = psi', diff = psi - psi', rPIE update of
//                      the object window (and the probe step), O written back
// so the exit wave is never stored and the object window is read twice and
// written once per position.  The scan index of the position comes from the
// device (order[iteration * nscan + k], iteration counter in device memory),
// so one sweep can be captured once and replayed.
#pragma once
#include "cdx_rfft.cuh"

namespace cdx {

struct PtyArgs {
  float2* W;               // work, column-tiled with width 2^tl
  float2* obj;             // object, row-major obj_rows x obj_cols
  const float2* probe;     // rows x cols
  float2* step;            // probe step accumulator (probe phase)
  const float* pats;       // nscan patterns, column-tiled, pat_stride floats apart
  const float* bs;         // beamstop, column-tiled, or null
  const int* order;        // scan index per slot (iteration * nscan + k)
  const int* iter;         // device iteration counter (relative to the run)
  const int2* win;         // window origin per scan index
  const float* scal;       // [0] max |P|^2, [1] object maximum (probe phase)
  const float2* tw;        // twiddles of the kernel's line length
  long long pat_stride;
  int rows, cols, obj_rows, obj_cols, tl, k, nscan, probe_phase;
  float norm;              // 1/sqrt(rows cols) (util/ptycho.cpp:439)
  float maximum;           // 0.95 * vars.scale, the saturation level of applyModAccurate
  float obj_step;          // rPIE step of the object: 1, or 0.5 in the probe phase
  float pss;               // probe step size 1/nscan
  int noise_proj;          // iteration >= 2000: applyMod (noise-tolerant) instead of applyModAccurate
  int noise_level;         // noiseLevel
  float ccd_scale;         // vars.scale = 1/exposure
  float rcolor;            // vars.rcolor
  int* err;                // bit 0: a bulk staging copy timed out
  float fresnel;           // isFresnel: the exit wave's Fresnel phase factor (0: off)
};

// multiplyFresnelPhase_Device at (row, col) of the rows x cols frame (cudaConfig.cu:1095-1101):
// v exp(i f ((row - rows/2)^2 + (col - cols/2)^2)) unless v is zero
__device__ __forceinline__ float2 pty_fresnel(float2 v, int row, int col, int rows, int cols, float f) {
  const int dx = row - (rows >> 1), dy = col - (cols >> 1);
  float s, c;
  sincosf(f * (float)(dx * dx + dy * dy), &s, &c);
  return (v.x != 0.f || v.y != 0.f) ? make_float2(v.x * c - v.y * s, v.x * s + v.y * c) : v;
}

constexpr float kPtyAlpha = 0.1f;   // ALPHA, src/gpu/ptycho.cu:5
constexpr float kPtyBeta = 0.5f;    // BETA, src/gpu/ptycho.cu:6

// rPIE (src/gpu/ptycho.cu:55-61): target -= conj(s) d * step / ((1-p)|s|^2 + p max(maxi, 1e-5)).
// The denominator is summed and divided in float (the reference: in double).
__device__ __forceinline__ float2 pty_rpie(float2 t, float2 s, float2 d, float maxi, float param, float stepsize) {
  float den = s.x * s.x + s.y * s.y;
  den = stepsize / ((1.f - param) * den + param * fmaxf(maxi, 1e-5f));
  t.x -= (s.x * d.x + s.y * d.y) * den;
  t.y -= (s.x * d.y - s.y * d.x) * den;
  return t;
}
// rPIE_step (src/gpu/ptycho.cu:62-68): -conj(s) d / ((1-p)|s|^2 + p max(maxi, 1e-5)).
__device__ __forceinline__ float2 pty_rpie_step(float2 s, float2 d, float maxi, float param) {
  float den = s.x * s.x + s.y * s.y;
  den = 1.f / ((1.f - param) * den + param * fmaxf(maxi, 1e-5f));
  return make_float2(-(s.x * d.x + s.y * d.y) * den, -(s.x * d.y - s.y * d.x) * den);
}

// applyModAccurate, 4-argument form (src/gpu/cdi.cu:351-388).
__device__ __forceinline__ float2 pty_modacc(float2 s, float inten, float bsv, bool has_bs, float norm,
                                             float maximum) {
  const float mod2 = fmaxf(0.f, inten);
  float rx = s.x, ry = s.y;
  if (norm != 1.f) { rx *= norm; ry *= norm; }
  if (has_bs && bsv > 0.5f) return make_float2(rx, ry);
  const float src = rx * rx + ry * ry;
  if (src == 0.f) return s;
  if (mod2 >= maximum && src >= mod2) return make_float2(rx, ry);
  const float sc = sqrtf(mod2 / src);
  return make_float2(sc * rx, sc * ry);
}

// applyMod, 5-argument form with bsnorm (src/gpu/cdi.cu:438-485): the
// noise-tolerant projection the reference switches to from iteration 2000.
__device__ __forceinline__ float2 pty_modnoise(float2 s, float inten, float bsv, bool has_bs, float norm, int noise,
                                               float scale, float rcolor) {
  float mod2 = fmaxf(0.f, inten);
  if (has_bs && bsv > 0.5f) return norm != 1.f ? make_float2(s.x * norm, s.y * norm) : s;
  float rx = s.x, ry = s.y;
  if (norm != 1.f) { rx *= norm; ry *= norm; }
  const float src = rx * rx + ry * ry;
  if (mod2 >= scale * 0.95f) mod2 = fmaxf(mod2, src);
  const float tol = sqrtf(noise + mod2 * rcolor / scale) * scale / rcolor;
  const float diff = mod2 - src;
  float val = mod2;
  if (diff > tol) val -= tol;
  else if (diff < -tol) val += tol;
  if (src == 0.f) return make_float2(val, 0.f);
  const float sc = sqrtf(fmaxf(val, 0.f) / src);
  return make_float2(sc * rx, sc * ry);
}

__device__ __forceinline__ long long pty_tiled(int r, int c, int rows, int tl) {
  return ((((long long)(c >> tl)) * rows + r) << tl) + (c & ((1 << tl) - 1));
}

// Row kernels stage the CTA's object-window rows and probe rows in shared
// memory with 8-byte cp.async (the window may start at any column; pixels
// outside the object are zero-filled), line stride N + 8 so the lines a warp
// reads together fall on different bank halves.
template <int N>
struct PtyRow {
  static constexpr int SN = N + 8;
  static constexpr int STAGE = 2 * Geom<N>::L * SN * (int)sizeof(float2);
  static constexpr int SMEM = Geom<N>::SMEM_LINES + STAGE;
};

template <int N>
__device__ __forceinline__ void pty_stage_rows(const PtyArgs& a, float2* o_s, float2* p_s, int row0, int nrows,
                                               int2 w) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T, SN = PtyRow<N>::SN;
  const long long OC = a.obj_cols;
  for (int e = threadIdx.x; e < L * N; e += T) {
    const int l = e / N, c = e - l * N;
    const int row = row0 + l;
    const bool rok = l < nrows;
    const int ox = w.x + row, oy = w.y + c;
    const bool inb = rok && ox >= 0 && ox < a.obj_rows && oy >= 0 && oy < a.obj_cols;
    cp_async8(o_s + l * SN + c, inb ? (const void*)(a.obj + ox * OC + oy) : (const void*)a.obj, inb);
    cp_async8(p_s + l * SN + c, rok ? (const void*)(a.probe + (long long)row * N + c) : (const void*)a.probe, rok);
  }
  cp_commit();
}

// ------------------------------------------------------- forward row pass
// FRES: isFresnel, a separate instantiation so the plain kernels carry no phase code
template <int N, bool FRES>
__global__ void __launch_bounds__(Geom<N>::T, Geom<N>::MINB) pty_fwd_rk(PtyArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L;
  using F0 = RFirst<N, 0>;
  using FL = RLast<N, 0>;
  constexpr int SN = PtyRow<N>::SN;
  extern __shared__ float2 smem[];
  pdl_wait_and_release();
  float2* o_s = smem + L * G::LD;
  float2* p_s = o_s + L * SN;
  const int row0 = blockIdx.x * L;
  const int nrows = min(L, a.rows - row0);
  const int cb = min(a.tl, rfft_cb_max<N>());
  const int si = a.order[*a.iter * a.nscan + a.k];
  pty_stage_rows<N>(a, o_s, p_s, row0, nrows, a.win[si]);
  cp_wait<0>();
  __syncthreads();
  float2 v0[F0::B][F0::R];
#pragma unroll
  for (int b = 0; b < F0::B; ++b) {
    int l, j;
    if (!bfly_of<N, F0::R>(b, cb, l, j)) continue;
#pragma unroll
    for (int r = 0; r < F0::R; ++r) {
      const int t = l * SN + j + r * F0::NR;   // multiply(esw, probe, window): zero outside the object
      v0[b][r] = cmul(p_s[t], o_s[t]);
      if constexpr (FRES) v0[b][r] = pty_fresnel(v0[b][r], row0 + l, j + r * F0::NR, a.rows, a.cols, a.fresnel);
    }
  }
  float2 v[FL::B][FL::R];
  rfft<N, 0, false>(v0, v, smem, a.tw, cb);
#pragma unroll
  for (int b = 0; b < FL::B; ++b) {
    int l, j;
    if (!bfly_of<N, FL::R>(b, cb, l, j) || l >= nrows) continue;
#pragma unroll
    for (int r = 0; r < FL::R; ++r) __stcg(a.W + pty_tiled(row0 + l, j + r * FL::NS, a.rows, a.tl), v[b][r]);
  }
}

// ------------------------------------------------------------ column pass
template <int N>
__global__ void __launch_bounds__(Geom<N>::T, RGeom<N>::MINB_COL) pty_col_rk(PtyArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L, T = G::T;
  using F0 = RFirst<N, 0>;
  using FL = RLast<N, 0>;
  using IL = RLast<N, 1>;
  extern __shared__ float2 smem[];
  pdl_wait_and_release();
  const int c0 = blockIdx.x * L;
  const int ncols = min(L, a.cols - c0);
  const long long tile = (long long)blockIdx.x * N * L;
  float* int_s = reinterpret_cast<float*>(smem + L * G::LD);
  float* bs_s = int_s + L * N;
  const int si = a.order[*a.iter * a.nscan + a.k];
  const float* pat = a.pats + si * a.pat_stride + tile;
  const bool has_bs = a.bs != nullptr;
  // the pattern tile (and the beamstop tile): contiguous L*N floats, bulk copies
  __shared__ uint64_t stage_bar;
  if constexpr (bulk_staging<N>()) {
    constexpr unsigned bytes = L * N * (unsigned)sizeof(float);
    if (threadIdx.x == 0) bulk_bar_init(&stage_bar);
    __syncthreads();
    if (threadIdx.x == 0) {
      bulk_expect(&stage_bar, bytes * (has_bs ? 2u : 1u));
      bulk_g2s(int_s, pat, bytes, &stage_bar);
      if (has_bs) bulk_g2s(bs_s, a.bs + tile, bytes, &stage_bar);
    }
  } else {
#pragma unroll 4
    for (int q = threadIdx.x; q < L * N / 4; q += T) {
      cp_async16(int_s + 4 * q, pat + 4 * q, true);
      if (has_bs) cp_async16(bs_s + 4 * q, a.bs + tile + 4 * q, true);
    }
    cp_commit();
  }
  float2 v0[F0::B][F0::R];
#pragma unroll
  for (int b = 0; b < F0::B; ++b) {
    int l, j;
    if (!bfly_of<N, F0::R>(b, 0, l, j)) continue;
#pragma unroll
    for (int r = 0; r < F0::R; ++r) v0[b][r] = __ldcg(a.W + tile + (long long)(j + r * F0::NR) * L + l);
  }
  float2 v[FL::B][FL::R];
  rfft<N, 0, false>(v0, v, smem, a.tw, 0);
  if constexpr (bulk_staging<N>()) bulk_wait(&stage_bar, a.err);
  else cp_wait<0>();
  __syncthreads();
#pragma unroll
  for (int b = 0; b < FL::B; ++b) {
    int l, j;
    if (!bfly_of<N, FL::R>(b, 0, l, j)) continue;
#pragma unroll
    for (int r = 0; r < FL::R; ++r) {
      const int t = (j + r * FL::NS) * L + l;
      const float bsv = has_bs ? bs_s[t] : 0.f;
      const float2 z = a.noise_proj ? pty_modnoise(v[b][r], int_s[t], bsv, has_bs, a.norm, a.noise_level,
                                                   a.ccd_scale, a.rcolor)
                                    : pty_modacc(v[b][r], int_s[t], bsv, has_bs, a.norm, a.maximum);
      v[b][r] = l < ncols ? z : make_float2(0.f, 0.f);
    }
  }
  float2 o[IL::B][IL::R];
  rfft<N, 1, true>(v, o, smem, a.tw, 0);
#pragma unroll
  for (int b = 0; b < IL::B; ++b) {
    int l, j;
    if (!bfly_of<N, IL::R>(b, 0, l, j)) continue;
#pragma unroll
    for (int r = 0; r < IL::R; ++r) __stcg(a.W + tile + (long long)(j + r * IL::NS) * L + l, o[b][r]);
  }
}

// -------------------------------------------------------- update row pass
template <int N, bool FRES>
__global__ void __launch_bounds__(Geom<N>::T, Geom<N>::MINB) pty_upd_rk(PtyArgs a) {
  using G = Geom<N>;
  constexpr int L = G::L;
  using F0 = RFirst<N, 0>;
  using FL = RLast<N, 0>;
  constexpr int SN = PtyRow<N>::SN;
  extern __shared__ float2 smem[];
  pdl_wait_and_release();
  float2* o_s = smem + L * G::LD;
  float2* p_s = o_s + L * SN;
  const int row0 = blockIdx.x * L;
  const int nrows = min(L, a.rows - row0);
  const int cb = min(a.tl, rfft_cb_max<N>());
  const int si = a.order[*a.iter * a.nscan + a.k];
  const int2 w = a.win[si];
  const long long OC = a.obj_cols;
  pty_stage_rows<N>(a, o_s, p_s, row0, nrows, w);   // lands during the inverse FFT
  float2 v0[F0::B][F0::R];
#pragma unroll
  for (int b = 0; b < F0::B; ++b) {
    int l, j;
    if (!bfly_of<N, F0::R>(b, cb, l, j)) continue;
#pragma unroll
    for (int r = 0; r < F0::R; ++r)
      v0[b][r] = l < nrows ? __ldcg(a.W + pty_tiled(row0 + l, j + r * F0::NR, a.rows, a.tl)) : make_float2(0.f, 0.f);
  }
  float2 v[FL::B][FL::R];
  rfft<N, 0, true>(v0, v, smem, a.tw, cb);
  cp_wait<0>();
  __syncthreads();
  const float pmax = a.scal[0], omax = a.scal[1];
#pragma unroll
  for (int b = 0; b < FL::B; ++b) {
    int l, j;
    if (!bfly_of<N, FL::R>(b, cb, l, j) || l >= nrows) continue;
#pragma unroll
    for (int r = 0; r < FL::R; ++r) {
      const int c = j + r * FL::NS, row = row0 + l;
      float2 pp = v[b][r];                       // IFFT, then applyNorm(Fn, norm)
      pp.x *= a.norm;
      pp.y *= a.norm;
      const int ox = w.x + row, oy = w.y + c;
      const bool inb = ox >= 0 && ox < a.obj_rows && oy >= 0 && oy < a.obj_cols;
      float2 o = o_s[l * SN + c];                // getWindow: zero outside the object
      const long long pi = (long long)row * N + c;
      const float2 p = p_s[l * SN + c];
      float2 d = cmul(p, o);                     // esw = P * O_window, then esw += Fn * (-1)
      if constexpr (FRES) d = pty_fresnel(d, row, c, a.rows, a.cols, a.fresnel);
      d.x -= pp.x;
      d.y -= pp.y;
      if constexpr (FRES) d = pty_fresnel(d, row, c, a.rows, a.cols, -a.fresnel);   // removeFresnelPhase
      o = pty_rpie(o, p, d, pmax, kPtyAlpha, a.obj_step);
      if (a.probe_phase) {
        const float2 st = pty_rpie_step(o, d, omax, kPtyBeta);
        float2 acc = a.step[pi];
        acc.x = acc.x + st.x * a.pss;
        acc.y = acc.y + st.y * a.pss;
        a.step[pi] = acc;
      }
      if (inb) a.obj[ox * OC + oy] = o;
    }
  }
}

// Launchers of the three kernels for line length N (host side).
template <int N>
cudaError_t pty_prepare() {
  using G = Geom<N>;
  cudaError_t e = cudaSuccess;
  const void* rows_k[] = {(const void*)pty_fwd_rk<N, false>, (const void*)pty_fwd_rk<N, true>,
                          (const void*)pty_upd_rk<N, false>, (const void*)pty_upd_rk<N, true>};
  for (const void* k : rows_k)
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, PtyRow<N>::SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(pty_col_rk<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             G::SMEM_LINES + 2 * G::L * N * (int)sizeof(float));
  return e;
}
template <int N>
cudaError_t pty_launch_fwd(const PtyArgs& a, cudaStream_t st) {
  using G = Geom<N>;
  const dim3 grid((a.rows + G::L - 1) / G::L);
  return a.fresnel != 0.f ? launch_pdl(pty_fwd_rk<N, true>, grid, G::T, PtyRow<N>::SMEM, st, a)
                          : launch_pdl(pty_fwd_rk<N, false>, grid, G::T, PtyRow<N>::SMEM, st, a);
}
template <int N>
cudaError_t pty_launch_upd(const PtyArgs& a, cudaStream_t st) {
  using G = Geom<N>;
  const dim3 grid((a.rows + G::L - 1) / G::L);
  return a.fresnel != 0.f ? launch_pdl(pty_upd_rk<N, true>, grid, G::T, PtyRow<N>::SMEM, st, a)
                          : launch_pdl(pty_upd_rk<N, false>, grid, G::T, PtyRow<N>::SMEM, st, a);
}
template <int N>
cudaError_t pty_launch_col(const PtyArgs& a, cudaStream_t st) {
  using G = Geom<N>;
  return launch_pdl(pty_col_rk<N>, dim3((a.cols + G::L - 1) / G::L), G::T,
                    G::SMEM_LINES + 2 * G::L * N * (int)sizeof(float), st, a);
}

#define CDX_PTY_INSTANTIATE(N)                                               \
  template cudaError_t pty_prepare<N>();                                     \
  template cudaError_t pty_launch_fwd<N>(const PtyArgs&, cudaStream_t);      \
  template cudaError_t pty_launch_upd<N>(const PtyArgs&, cudaStream_t);      \
  template cudaError_t pty_launch_col<N>(const PtyArgs&, cudaStream_t);

}  // namespace cdx
