/* C ABI of the GB300 ptychographic reconstruction (rPIE object and probe
 * updates with mPIE momentum): the reference's ptycho::iterate
 * (util/ptycho.cpp:429-736) and the kernels it calls (src/gpu/ptycho.cu:9-113,
 * applyModAccurate src/gpu/cdi.cu:351-388, the angular-spectrum propagator
 * src/post_gpu/propagator.cc:31-49), plus the set-up steps of its driver
 * (initObject util/ptycho.cpp:363-369, the noise-free part of createPattern
 * 310-359).
 *
 * The reference keeps this path in an executable (util/ptycho.cpp main) that
 * owns its buffers through the process-wide memory pool; here a handle owns
 * them.  Every call returns CDX_OK (0) or a CDX_ERR_* code of cdx.h with the
 * message in cdx_last_error(); no call aborts the process.  Host pointers
 * are plain row-major arrays; complex values are interleaved float pairs
 * (the reference's complexFormat).
 */
#ifndef CDX_PTYCHO_H
#define CDX_PTYCHO_H

#include "cdx.h"

#ifdef __cplusplus
extern "C" {
#endif
#pragma GCC visibility push(default)

typedef struct cdx_pty cdx_pty;

/* The fields ptycho::iterate reads (include/readConfig.hpp:25-35, where the
 * real-valued ones are double) and the sizes the ptycho program derives. */
typedef struct cdx_pty_params {
  int rows, cols;          /* probe and pattern size (row, column); 2^a 3^b in [16, 4096] */
  int obj_rows, obj_cols;  /* object size (row_O, column_O) */
  int nscan;               /* scan positions */
  double lambda;           /* wavelength */
  double d;                /* sample-detector distance */
  double dpupil;           /* pupil-sample distance (propagate_pupil.distance) */
  double pixelsize;        /* detector pixel size */
  double pupil_size;       /* pupil diameter in pixels (pupilSize) */
  double exposure;         /* patterns are stored scaled by 1/exposure */
  int mpie;                /* momentum step after each sweep (mPIE, default 1) */
  int use_bs;              /* beamstop of radius beam_stop_size at the pattern centre (useBS) */
  int beam_stop_size;
  int noise_level;         /* noiseLevel: tolerance of the modulus projection from iteration 2000 */
  double position_uncertainty; /* positionUncertainty: > 0 refines the scan positions every 20 sweeps from
                                  500 (util/ptycho.cpp:511-585); the object is shifted by FFT, so its sizes
                                  must then be 2^a 3^b in [16, 4096] */
  int zernike_iter;        /* zernikeIter: before it the object takes a FISTA (TV) step each sweep and,
                              every tenth sweep, the probe a momentum step (with mPIE) and, from
                              iteration 400, the Zernike pupil fit (861 modes up to order 40) in place of
                              the pupil disk (util/ptycho.cpp:484, 617-626, 665-671) */
  int is_fresnel;          /* isFresnel: the exit wave times the Fresnel phase of distance d before
                              its transform, the difference of exit waves times its inverse after
                              (util/ptycho.cpp:323-326, 526-528, 551; propagator.cc:15-20) */
} cdx_pty_params;

/* Defaults of readConfig (include/readConfig.hpp): mPIE 1, pupilSize 500,
 * beamStopSize 5, exposure 1; sizes and optics are the caller's. */
int cdx_pty_params_default(cdx_pty_params* p);

/* Allocates the object, probe, pattern stack, work buffers and device
 * scalars on the current device.  `stream` may be NULL (a stream of its own). */
int cdx_pty_create(const cdx_pty_params* p, void* stream, cdx_pty** out);
int cdx_pty_destroy(cdx_pty* t);

/* Scan positions in object pixels (scanposx/scanposy, util/ptycho.cpp:46-47):
 * the window of position i starts at round(x_i), round(y_i); the overlap mask
 * takes them truncated, as the reference's int parameters do. */
int cdx_pty_set_scan(cdx_pty* t, const float* posx, const float* posy);

/* nscan stacked rows x cols patterns in FFT (unshifted) order, scaled by
 * 1/exposure, as ptycho::patterns holds them (util/ptycho.cpp:355-358, 713-716). */
int cdx_pty_set_patterns(cdx_pty* t, const float* patterns);
int cdx_pty_get_patterns(cdx_pty* t, float* patterns);

int cdx_pty_set_object(cdx_pty* t, const float* obj);     /* obj_rows x obj_cols complex */
int cdx_pty_get_object(cdx_pty* t, float* obj);
int cdx_pty_set_probe(cdx_pty* t, const float* probe);    /* rows x cols complex, sample plane */
int cdx_pty_get_probe(cdx_pty* t, float* probe);
/* The probe back-propagated to the pupil plane, which is what the reference
 * leaves in pupilpatternWave after iterate() (util/ptycho.cpp:705). */
int cdx_pty_get_pupil(cdx_pty* t, float* pupil);
/* The probe from a pupil-plane field: probe = angularSpectrumPropagate(pupil)
 * by dpupil (what readPupilAndObject does with the pupil image,
 * util/ptycho.cpp:275-287). */
int cdx_pty_set_pupil(cdx_pty* t, const float* pupil);

/* initObject (util/ptycho.cpp:363-369): the object set to unit modulus with a
 * uniform random phase (a counter-based generator keyed by seed and pixel,
 * not curand MRG32k3a), the probe to the pupil disk of pupil_size
 * (pupilFunc, src/gpu/ptycho.cu:123-130) propagated by dpupil. */
int cdx_pty_init_object(cdx_pty* t, unsigned long long seed);

/* createPattern without detector noise (util/ptycho.cpp:310-359): pattern i =
 * |FFT(probe * window_i(object))|^2 / (rows cols) (zero under the beamstop with
 * use_bs), from the current object and probe, stored as the context's patterns. */
int cdx_pty_simulate(cdx_pty* t);
/* createPattern with simCCDbit: the same intensities recorded by ccdRecord
 * (Poisson(noise_level + rcolor I exposure), clamped below rcolor, minus
 * noise_level, / rcolor; src/gpu/cdi.cu:260-266) and scaled by 1/exposure;
 * counter-based random numbers keyed by seed, position and pixel. */
int cdx_pty_simulate_ccd(cdx_pty* t, unsigned long long seed);

/* ptycho::iterate: n_iter sweeps starting at iteration index first_iter
 * (the reference always starts at 0; from index 400 the probe is updated and
 * constrained, from 2000 the modulus projection is the noise-tolerant
 * applyMod).  orders: n_iter x nscan scan indices, one permutation per
 * sweep, or NULL to draw them as the reference does (shuffle_array with a
 * rand() stream seeded by `seed`, the generator of the C library restated).
 * Fresh per-call state as in the reference (zero momentum history and probe
 * step).  From iteration 500 the reference refines the scan positions every
 * 20 sweeps; with position_uncertainty = 0 (its default) that step leaves
 * the positions at zero shift and the object unchanged up to the rounding of
 * an FFT round trip, which is not repeated here; with position_uncertainty > 0
 * the shifts are refined (zero at the start of each call) and the object is
 * shifted by their mean (object sizes 2^a 3^b, else CDX_ERR_SIZE for runs past
 * iteration 500).  The final
 * object has its global phase removed (util/ptycho.cpp:731-735). */
int cdx_pty_iterate(cdx_pty* t, int first_iter, int n_iter, const int* orders, unsigned int seed);

/* Device time of the last cdx_pty_iterate in milliseconds. */
int cdx_pty_last_ms(cdx_pty* t, float* ms);

/* The scan orders the reference's rand()-driven shuffle gives for a seed
 * (n_iter x nscan), for callers that want to log or replay them. */
int cdx_pty_scan_orders(int nscan, int n_iter, unsigned int seed, int* orders);

#pragma GCC visibility pop
#ifdef __cplusplus
}
#endif
#endif
