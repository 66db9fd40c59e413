/*
 * cunfft_typedefs.h -- types of the CUNFFT drop-in plan ABI.
 *
 * Field order and types of kdata and cunfft_plan are those of the reference
 * (src/cunfft_typedefs.h:98-178) under its committed configuration
 * (src/config.h: CUNFFT_DOUBLE_PRECISION, LARGE_INPUT), so that programs and
 * language bindings written against CUNFFT keep working unchanged: the caller
 * owns the cunfft_plan storage, reads and writes plan.x / plan.f_hat / plan.f on
 * the host, and the library fills the remaining members.  Extra state of this
 * library lives in a side table keyed by the plan's address; the struct does
 * not grow.
 */
#ifndef CUNFFT_TYPEDEFS_H_
#define CUNFFT_TYPEDEFS_H_

#include <stddef.h>
#include <cuComplex.h>
#include <cufft.h>

#include "config.h"
#include "timeMeasurement.h"

/** Size of the filter window, 2m+2 taps per dimension. */
#define FILTER_SIZE ((2 * CUT_OFF) + 2)
/** Maximum dimension supported by the plan API. */
#define MAX_DIM 3
/** Maximum cut-off parameter. */
#define MAX_FILTER_RADIUS 50

/** Plan flags (src/cunfft_typedefs.h:47-53). */
#define CUFFT_INIT  (1U << 0)
#define CUFFT_BOTH  (1U << 1)
#define CUFFT_FORW  (1U << 2)
#define CUFFT_BACKW (1U << 3)

/** Complex and real types: double precision, as the committed configuration. */
typedef cuDoubleComplex gpuComplex;
typedef double dTyp;
/** Index types: ptrdiff_t, as LARGE_INPUT. */
typedef ptrdiff_t uint_t;
typedef ptrdiff_t sint_t;
#define PRINT_FORMAT "%ld"
#define PRINT(V, F) printf(#V " = " F, V)

/** Transform properties (reference: uploaded to __constant__ memory; here
 *  only filled by setProperties for callers that read it). */
typedef struct {
  uint_t N[MAX_DIM];      /**< bandwidths */
  uint_t n[MAX_DIM];      /**< oversampled FFT lengths */
  double b[MAX_DIM];      /**< Gaussian shape b_t = 2 sigma/(2 sigma - 1) * m/pi */
  double bsqrt[MAX_DIM];  /**< sqrt(b_t) */
  double fac[MAX_DIM];    /**< pi^2 b_t / n_t^2 */
  double sigma[MAX_DIM];  /**< oversampling factor n_t / N_t */
} kdata;

/** The plan (field order and types of the reference). */
typedef struct {
  uint_t N_total;        /**< number of Fourier coefficients */
  uint_t M_total;        /**< number of nodes */
  int d;                 /**< dimension */
  uint_t *N;             /**< bandwidths [d] */
  dTyp *x;               /**< host nodes [M_total*d], x[j*d+t] in [-0.5, 0.5) */
  gpuComplex *f_hat;     /**< host coefficients [N_total], row-major, dim 0 slowest */
  gpuComplex *f;         /**< host samples [M_total] */
  double *sigma;         /**< oversampling factors [d] */
  uint_t *n;             /**< FFT lengths [d] */
  uint_t n_total;        /**< prod n */
  int m;                 /**< window cut-off */
  double *b;             /**< window shapes [d] */
  gpuComplex *g;         /**< host copy of the oversampled grid [n_total] */
  gpuComplex *g_hat;     /**< unused (kept for layout) */
  double *fg_exp_l_cpu;  /**< fast-Gaussian-gridding table exp(-l^2/b_t), FILTER_SIZE per dim */
  gpuComplex *g_gpu;     /**< device oversampled grid */
  gpuComplex *fhat_gpu;  /**< device coefficients */
  dTyp *x_gpu;           /**< device nodes */
  gpuComplex *f_gpu;     /**< device samples */
  cufftHandle fft_forward;   /**< cuFFT plan used by the forward transform */
  cufftHandle fft_backward;  /**< cuFFT plan used by the adjoint transform */
  NFFTTimeSpec CUNFFTTimes;  /**< per-step times of the last call (seconds) */
  unsigned flags;            /**< CUFFT_INIT | CUFFT_BOTH | ... */
} cunfft_plan;

#endif /* CUNFFT_TYPEDEFS_H_ */
