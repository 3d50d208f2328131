// Host stand-in for the GSL spline calls of src/post_gpu/misc.cc (spectrum
// resampling, outside the ptychography path): every call aborts.
#pragma once
#include <cstdlib>
struct gsl_interp_accel { int d; };
struct gsl_spline { int d; };
struct gsl_interp_type { int d; };
static const gsl_interp_type* gsl_interp_cspline = nullptr;
inline gsl_interp_accel* gsl_interp_accel_alloc() { abort(); }
inline gsl_spline* gsl_spline_alloc(const gsl_interp_type*, size_t) { abort(); }
inline int gsl_spline_init(gsl_spline*, const double*, const double*, size_t) { abort(); }
inline double gsl_spline_eval(const gsl_spline*, double, gsl_interp_accel*) { abort(); }
inline void gsl_spline_free(gsl_spline*) {}
inline void gsl_interp_accel_free(gsl_interp_accel*) {}
