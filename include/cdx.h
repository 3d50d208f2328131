/* cdx.h -- C ABI of the GB300-native CDI phase-retrieval path.
 *
 * Replaces the GPU side of liboyang0112/CDIxx's CDI iteration: the cuFFT
 * wrapper, the modulus projections, the real-space updates and the
 * shrinkwrap of CDI::phaseRetrieve.  Plain pointers and sizes only; every
 * call returns a status code (CDX_OK == 0) instead of aborting, and
 * cdx_last_error() describes the last failure of the calling thread.
 *
 * Complex arrays are interleaved float pairs (the reference's
 * complexFormat = _Complex float, include/format.hpp:25-26), row-major,
 * rows x cols per pattern, patterns back to back.  Fourier-space arrays are
 * in FFT (unshifted) order, as the reference keeps patternData/patternWave.
 * `where` selects host (CDX_HOST) or device (CDX_DEVICE) memory for a buffer.
 */
#ifndef CDX_H
#define CDX_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

enum {
  CDX_OK = 0,
  CDX_ERR_ARG = 1,       /* bad argument (null pointer, index out of range) */
  CDX_ERR_SIZE = 2,      /* unsupported pattern size (rows, cols must be 2^a 3^b in [16, 4096]) */
  CDX_ERR_CUDA = 3,      /* a CUDA call failed; cdx_last_error() has the CUDA message */
  CDX_ERR_ALGO = 4,      /* algorithm string rejected (unknown token, TV step) */
  CDX_ERR_STATE = 5,     /* call order: no pattern / no initial iterate yet */
  CDX_ERR_IO = 6,        /* .bin file missing, short or of the wrong type */
  CDX_ERR_NOMEM = 7,     /* device allocation failed */
  CDX_ERR_CONFIG = 8,    /* config file could not be parsed */
  CDX_ERR_NOLIB = 9      /* the CUDA device or kernels are unavailable */
};
enum { CDX_HOST = 0, CDX_DEVICE = 1 };
enum { CDX_FFT_ORDER = 0, CDX_CENTERED = 1 };

/* Algorithm codes = the reference's Algorithm enum (include/format.hpp:22). */
enum { CDX_RAAR = 0, CDX_ER = 1, CDX_POSER = 2, CDX_HIO = 3, CDX_POSHIO = 4, CDX_FHIO = 5,
       CDX_SHRINKWRAP = 6, CDX_XCORRELATION = 7, CDX_KKT = 8, CDX_TV = 9 };

/* Shrinkwrap kernels. */
enum {
  CDX_SHRINK_FOURIER = 0,  /* CDI::phaseRetrieve (cdi.cc:326-341): |IFFT(G_sf Psi)|^2, sf = (rows/4)/g,
                              g = sigma0 then *= decay while > sigma_min; thr = min(max, 5 avg0) * shrinkThreshold */
  CDX_SHRINK_SPATIAL = 1   /* holo::iterate (holo.cc:125-148): G_sigma (*) |rho|^2 in pixels,
                              sigma = sigma0 then *= decay while > sigma_min; thr = max * shrinkThreshold */
};

typedef struct cdx_params {
  int rows, cols;            /* pattern size (row, column of the reference) */
  int batch;                 /* patterns of this size held by the context */
  float beta;                /* vars.beta_HIO (src/gpu/cdi.cu:22; the reference fixes it at 1) */
  float shrink_threshold;    /* shrinkThreshold */
  float oversampling_spt;    /* oversampling_spt: initial rect support (cdi.cc:240-251) */
  float exposure;            /* exposure: vars.scale = 1/exposure (cdi.cc:52) */
  int rcolor;                /* vars.rcolor (65535) */
  int sim_ccd_bit;           /* simCCDbit: applyMod instead of applyModAbs (cdi.cc:349-350) */
  int noise_level;           /* noiseLevel */
  int shrink_mode;           /* CDX_SHRINK_* */
  float sigma0, sigma_min, sigma_decay;  /* shrinkwrap width schedule (defaults 3, 2, 0.99) */
  int use_graph;             /* capture each cdx_run in a CUDA graph (default 1) */
  int rf_every;              /* compute the R-factor every k iterations inside the loop (0 = only at the end) */
  float stop_rfactor;        /* with rf_every > 0: a pattern whose R-factor <= stop_rfactor finishes its
                                iteration and then freezes (its kernels return at once); 0 = never */
  int fft_mode;              /* CDX_FFT_FP32 (default) or CDX_FFT_TC_BF16 */
  int prtf_iter;             /* prtfIter: from this step on (the step counter of phaseRetrieve, shrinkwraps
                                included) accumulate the phase-retrieval transfer function; -1 = off (default) */
  int autotune;              /* 1: before the first run of a size, time the launch variants of the iteration
                                (programmatic dependent launch on/off x row-pass butterfly chunk width) on the
                                context's own data and keep the fastest (cached per device, size and batch for
                                the process); 0 (default): the per-length defaults */
  int plateau_iters;         /* with rf_every > 0: a pattern whose lowest in-loop R-factor has not fallen by
                                a factor (1 - plateau_tol) within this many iterations freezes (0 = off) */
  float plateau_tol;         /* relative improvement that counts for plateau_iters (default 0.01) */
} cdx_params;

/* FFT arithmetic.  CDX_FFT_TC_BF16: the radix-16 passes run as tcgen05
 * tensor-core MMAs (accumulator in TMEM) with BF16 head/tail operands and FP32
 * accumulation (relative error per 2-D transform ~1e-5 instead of ~1.5e-7);
 * CDX_FFT_TC_MMA: the same split product on warp-level mma.sync.  No
 * reference counterpart. */
enum { CDX_FFT_FP32 = 0, CDX_FFT_TC_BF16 = 1, CDX_FFT_TC_MMA = 2 };

typedef struct cdx_stats {
  int steps;                 /* algorithm steps executed (iterations + shrinkwraps) */
  int iterations;            /* projection iterations */
  int shrinkwraps;
  double residual;           /* pattern 0: the reference's residual (cdi.cc:413-421) */
  double rfactor;            /* pattern 0: sum| |Psi|-sqrt(I) | / sum sqrt(I) of the final Psi */
  float threshold;           /* pattern 0: vars.threshold after the run */
  int flags;                 /* pattern 0: bit 0 = a shrinkwrap saw max ~ 0 or NaN (cdi.cc:334-337) */
  double gpu_ms;             /* device time of the run (CUDA events) */
  int launches;              /* kernels the run enqueued */
  int converged_iter;        /* iterations run before the pattern froze at stop_rfactor or on a plateau
                                (-1: never); flags bit 3 set when the plateau froze it */
  double rfactor_min;        /* lowest R-factor of the in-loop checks (rf_every); +inf without any */
} cdx_stats;

typedef struct cdx_ctx cdx_ctx;

/* ---------------------------------------------------------------- context */
/* Fill *p with the reference's defaults (readConfig.hpp:25-35 plus beta = 1). */
int cdx_params_default(cdx_params* p);
/* Allocate a context for `p->batch` patterns of p->rows x p->cols on the
 * current device.  `stream` is a cudaStream_t (NULL: the context creates one).
 * Replaces CDI::allocateMem / init_fft / init_cuda_image (cdi.cc:42-61,
 * cudaConfig.cu:137-159, cdi.cu:16-30). */
int cdx_create(const cdx_params* p, void* stream, cdx_ctx** out);
int cdx_destroy(cdx_ctx* ctx);
int cdx_get_params(const cdx_ctx* ctx, cdx_params* out);
/* Device pointers of the context's arrays (the CDI class exposes them as
 * patternData, patternWave, objectWave, support).  Any may be NULL. */
int cdx_device_arrays(cdx_ctx* ctx, float** pattern, void** fourier, void** object, float** support);

/* ---------------------------------------------------------------- inputs */
/* Pattern intensity of pattern `idx` (rows x cols floats), multiplied by
 * `scale` on the device (applyNorm(patternData, 1/exposure), cdi.cc:106).
 * layout CDX_CENTERED applies cudaConvertFO first (cdi.cc:105).  Also resets
 * the support of that pattern to the rect of oversampling_spt. */
int cdx_set_pattern(cdx_ctx* ctx, int idx, const float* intensity, int where, int layout, float scale);
/* Optional beamstop (useBS; cdi.cc:131-148), same layout rules, NULL clears it. */
int cdx_set_beamstop(cdx_ctx* ctx, int idx, const float* bs, int where, int layout);
/* Restart iterate Psi0 (prepareIter with restart, cdi.cc:201-227):
 * rho0 = IFFT(Psi0)/sqrt(N).  Also resets the support to the rect (initSupport). */
int cdx_set_initial(cdx_ctx* ctx, int idx, const float* psi0, int where);
/* Random-phase start for every pattern (cdi.cc:222-227): Psi0 = sqrt(I) e^{i pi b}. */
int cdx_random_start(cdx_ctx* ctx, unsigned long long seed);
/* Float support of pattern idx (inside = value > current threshold). */
int cdx_set_support(cdx_ctx* ctx, int idx, const float* support, int where);
/* Stop R-factor of pattern idx alone (0: the context's stop_rfactor); with
 * rf_every > 0 the pattern freezes once its in-loop R-factor <= stop, e.g. a
 * noise-aware stop just above that pattern's Poisson floor.  No reference
 * counterpart (the reference has no in-loop stop). */
int cdx_set_stop_rfactor(cdx_ctx* ctx, int idx, double stop);

/* ---------------------------------------------------------------- the loop */
/* CDI::phaseRetrieve (cdi.cc:297-449) on every pattern of the context, with
 * the reference's algorithm grammar (readConfig.cc:82-163), e.g.
 * "100*(3*POSHIO+20*RAAR+1*POSHIO+1*shrinkWrap)+20*RAAR+1*ER".
 * Nested parentheses are accepted too.  Ends with rho scaled by sqrt(N), Psi
 * = FFT(rho) and the residual.  Synchronises the context's stream. */
int cdx_run(cdx_ctx* ctx, const char* algorithm, cdx_stats* stats);
/* Same without the final synchronisation or statistics (device timing). */
int cdx_run_async(cdx_ctx* ctx, const char* algorithm);
/* Statistics of pattern idx after a run (synchronises). */
int cdx_get_stats(cdx_ctx* ctx, int idx, cdx_stats* stats);

/* ---------------------------------------------------------------- uneven batches */
/* A group runs phaseRetrieve on several contexts (typically one per pattern
 * size, each holding a batch of equal-size patterns) as ONE CUDA graph with a
 * branch per context, so patterns of uneven sizes run in a single launch.  No
 * reference counterpart (the reference runs one pattern at a time).  The
 * contexts must use distinct streams (created by cdx_create with stream NULL)
 * and stay alive while the group exists. */
typedef struct cdx_group cdx_group;
int cdx_group_create(cdx_ctx* const* ctxs, int n, cdx_group** out);
/* Runs `algorithm` on every context; synchronises; *gpu_ms gets the graph's
 * device time (may be NULL).  Per-pattern results: cdx_get_stats / cdx_get_*. */
int cdx_group_run(cdx_group* g, const char* algorithm, double* gpu_ms);
/* Branch order of the group's graph: 0 (default) the contexts one after
 * another, nonzero side by side.  Each size's pass kernels already fill the GPU
 * from 192^2 x 100 up, and side-by-side branches then slow one another (the
 * 512-pattern uneven batch: 648 ms side by side, 620 ms one after another);
 * batches too small to fill the GPU gain from running side by side.  The next
 * cdx_group_run captures the graph again. */
int cdx_group_set_concurrent(cdx_group* g, int concurrent);
int cdx_group_destroy(cdx_group* g);

/* ---------------------------------------------------------------- outputs */
int cdx_get_object(cdx_ctx* ctx, int idx, float* out, int where);   /* objectWave (complex) */
int cdx_get_fourier(cdx_ctx* ctx, int idx, float* out, int where);  /* patternWave (complex) */
int cdx_get_support(cdx_ctx* ctx, int idx, float* out, int where);  /* support (float field) */
/* PRTF of the last run (cdi.cc:355-380, 424-440): rows/2 floats, radius r =
 * the angular sum of |<P_M Psi e^{i phi}>| over the steps from prtf_iter on,
 * divided by the angular sum of the |P_M Psi| > 1e-6 mask at prtf_iter (the
 * prtf.txt column).  CDX_ERR_STATE when the run did not reach prtf_iter. */
int cdx_get_prtf(cdx_ctx* ctx, int idx, float* out, int where);
/* The launch variant the iteration uses (autotune): *pdl bit 0 = the column
 * pass is a programmatic dependent launch, bit 1 = the row pass (-1: the
 * per-length defaults); *row_chunk = butterfly chunk bits of the row pass
 * (-1: the default); `report` (may be NULL) receives the timings the
 * autotuner measured, one "pdl_col=<0|1> pdl_row=<0|1> chunk=<k>: <us> us"
 * line per variant ("cached" / "loaded" when the decision was reused). */
int cdx_get_tuning(cdx_ctx* ctx, int* pdl, int* row_chunk, char* report, int cap);
/* The autotuner's decisions as a JSON file, keyed by device name, rows, cols
 * and batch: save writes every decision of this process (and every loaded
 * one); load reads a file written by save (*count = its entries, may be NULL),
 * and contexts created afterwards on a device of that name take those
 * decisions instead of timing the variants. */
int cdx_tuning_save(const char* path);
int cdx_tuning_load(const char* path, int* count);

/* ---------------------------------------------------------------- one call, host buffers */
/* Whole path for one pattern with HOST buffers: create, set pattern, set
 * Psi0 (or a random start when psi0 is NULL), run, copy rho/Psi/support
 * back.  Outputs may be NULL.  The call keeps its context (device arrays and
 * the CUDA graph of the last algorithm) for the next call with the same
 * parameters on the same device, returned to the state of a new context
 * before reuse (the reference keeps its memory pool and cuFFT plan for the
 * whole process, memManager.cc, cudaConfig.cu:137-159); concurrent calls
 * each get their own.  cdx_release_host_cache frees the kept context; call it
 * before cudaDeviceReset, which would leave the kept context's memory invalid. */
int cdx_phase_retrieve_host(const cdx_params* p, const char* algorithm, const float* intensity,
                            const float* psi0, unsigned long long seed, float* rho_out, float* psi_out,
                            float* support_out, cdx_stats* stats);
int cdx_release_host_cache(void);

/* ---------------------------------------------------------------- primitives (device pointers) */
/* myFFT / myIFFT (cudaConfig.cu:175-180): unnormalised 2-D C2C transform of
 * `batch` patterns, in place allowed.  inverse != 0 uses exp(+2 pi i). */
int cdx_fft2(const void* in, void* out, int rows, int cols, int batch, int inverse, void* stream);
/* applyPoissonNoise_WO (src/gpu/cdi.cu:291-296), the simulation's detector
 * model (simCCDbit, cdi.cc:191-193): on `count` floats of a DEVICE pattern,
 * I <- s (trunc(I rcolor / s) + Poisson(noise_level) - noise_level) / rcolor
 * with s = 1/exposure (vars.scale).  Random numbers are counter based (seed,
 * pixel index), not the reference's curand MRG32k3a states. */
int cdx_ccd_noise(float* pattern, long long count, float noise_level, float exposure, int rcolor,
                  unsigned long long seed, void* stream);
/* propagator::multiplyFresnelPhase / removeFresnelPhase (src/post_gpu/propagator.cc:15-20):
 * the phase factor pi lambda d / (pixelsize rows)^2 of the propagator's float members
 * (negated when `remove`), and multiplyFresnelPhase_Device (cudaConfig.cu:1095-1101) on a
 * DEVICE field of `batch` rows x cols complex images: a <- a exp(i factor ((x - rows/2)^2 +
 * (y - cols/2)^2)) on the entries that are not zero. */
float cdx_fresnel_factor(double lambda, double distance, double pixelsize, int rows, int remove);
int cdx_fresnel_phase(void* field, int rows, int cols, int batch, float factor, void* stream);
/* ccdRecord(data, wave, noiseLevel, state, exposure) (src/gpu/cdi.cu:260-266), the detector
 * model of ptycho::createPattern with simCCDbit: on `count` floats of a DEVICE pattern,
 * I <- (min(Poisson(noiseLevel + rcolor I exposure), rcolor - 1) - noiseLevel) / rcolor * post.
 * Counter-based random numbers (seed, element index), not curand MRG32k3a states. */
int cdx_ccd_record(float* pattern, long long count, int noise_level, float exposure, int rcolor, float post,
                   unsigned long long seed, void* stream);
/* cdx_fft2 with the FFT arithmetic chosen by fft_mode (CDX_FFT_*). */
int cdx_fft2_ex(const void* in, void* out, int rows, int cols, int batch, int inverse, int fft_mode, void* stream);
/* applyModAbs(source, target) with state NULL (cudaConfig.cu:827-841). */
int cdx_apply_mod_abs(void* psi, const float* intensity, long long n, void* stream);
/* applyMod(source, target, bs, noiseLevel) (cdi.cu:438-485); scale = vars.scale. */
int cdx_apply_mod(void* psi, const float* intensity, const float* beamstop, int noise_level, float scale,
                  int rcolor, long long n, void* stream);
/* applySupport(gkp1, gkprime, algo, spt) (cdi.cc:25-36, cdi.cu:518-616). */
int cdx_apply_support(void* rho, const void* rho_prime, const float* support, float threshold, float beta,
                      int algo, long long n, void* stream);
/* cudaConvertFO for complex or real arrays (cudaConfig.cu:202-216). */
int cdx_convert_fo(const void* in, void* out, int rows, int cols, int batch, int is_complex, void* stream);

/* ---------------------------------------------------------------- no device allocation */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: a detector's acquisition loop that cannot afford the device-wide
 * synchronisation cudaMalloc/cudaFree bring between frames, or a plugin whose
 * host application owns the whole device-memory budget.
 *
 * cdx_iterate_noalloc runs `iterations` fused iterations of update `algo`
 * (CDX_HIO, CDX_RAAR, CDX_ER, ...; no shrinkwrap) on one rows x cols pattern,
 * with the projection of applyModAbs: the same kernels and results as
 * cdx_set_pattern + cdx_set_initial + cdx_set_support + cdx_run("<n>*ALGO").
 * The caller passes DEVICE buffers, each starting on a 16-byte boundary:
 * intensity (rows*cols floats, FFT order), support (floats; inside = value >
 * threshold), psi0 (restart iterate, complex) and the outputs rho_out
 * (object, scaled like phaseRetrieve leaves it) and psi_out (final Fourier
 * iterate).  rho_out must not overlap any other buffer; psi_out must not
 * overlap intensity, support or rho_out, and may be psi0 itself (CDX_ERR_ARG
 * otherwise).  The call allocates nothing: its scratch is a static device
 * array of CDX_NOALLOC_SCRATCH_BYTES inside this library, held by every GPU
 * that loads the library until the process exits, which bounds patterns to
 * CDX_NOALLOC_MAX_PIXELS pixels (512 x 512; larger sizes return
 * CDX_ERR_SIZE).  All calls share that array and it keeps the last call's
 * contents (each call clears what it uses): calls that overlap on the GPU
 * race.  The first call on a device is its set-up: it looks the array up on
 * that device and copies the FFT twiddle tables in with a blocking copy; make
 * it before any stream capture.  Every later call only queues work on
 * `stream` and returns without waiting for it.  If a kernel's bounded
 * staging wait runs out (a guard against a hang), rho_out and psi_out are
 * filled with NaN. */
#define CDX_NOALLOC_MAX_PIXELS (512 * 512)
#define CDX_NOALLOC_SCRATCH_BYTES (6u << 20)
int cdx_iterate_noalloc(int rows, int cols, int algo, float beta, int iterations, const float* intensity,
                        const float* support, float threshold, const void* psi0, void* rho_out, void* psi_out,
                        void* stream);

/* ---------------------------------------------------------------- helpers */
/* AlgoParser (readConfig.cc:82-163): expand `algorithm` into step codes.
 * Writes up to `cap` codes to `out` (may be NULL) and the total to *count. */
int cdx_algo_expand(const char* algorithm, int* out, int cap, int* count);
/* .bin image files (imgio.c:23-43, 223-243).  cdx_read_bin with data NULL
 * returns the header only; *is_complex set from the file type. */
int cdx_read_bin(const char* path, int* rows, int* cols, int* is_complex, float* data, size_t cap_floats);
int cdx_write_bin(const char* path, const float* data, int rows, int cols, int is_complex);
/* Lengths the kernels support (2^a 3^b, 16..4096). */
int cdx_size_supported(int n);
const char* cdx_last_error(void);
const char* cdx_version(void);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif /* CDX_H */
