/*
 * cunfft_util.h -- driver utilities of the CUNFFT plan API.
 *
 * The subset of the reference's utility API (src/cunfft_util.h) that its
 * drivers call (src/simpleTest.cpp, Tests/Scripts/simpleTest.cpp): example
 * data from drand48, the relative l_inf error norm, and console output.  The
 * reference's DEBUG error macros exit the process; here cudaVerify and
 * cufftVerify print the failure and continue, matching the library's
 * no-exit policy.
 */
#ifndef CUNFFTUTIL_H_
#define CUNFFTUTIL_H_

#include <stdio.h>
#include <stdlib.h>
#include <math.h>

#include "cunfft.h"

#ifdef __cplusplus
extern "C" {
#endif

#define K2PI 6.2831853071795864769252867665590057683943387987502

/** Print the step times of a plan divided by tfac (reference src/cunfft_util.h:94). */
void showTimes(NFFTTimeSpec *times, int tfac);
/** Print device memory statistics; returns free bytes (reference src/cunfft_util.h:167). */
unsigned long getGPUMemProps_ToStdout(void);
/** Print the host memory a plan needs (reference src/cunfft_util.h:174). */
void showCPUMemUse(cunfft_plan *p);
/** Print the first n entries (reference src/cunfft_util.h:187, :197). */
void showCoeff_double(const dTyp *x, int n, const char *text);
void showCoeff_cuComplex(const gpuComplex *x, int n, const char *text);
/** Product of the first d entries / next power of two >= N (reference src/cunfft_util.h:221, :229). */
uint_t prod_int(uint_t *vec, int d);
uint_t next_power_of_2(uint_t N);
/** Coefficient generators (reference src/cunfft_util.h:240-254, src/cuda_util.cpp:194-222). */
void createFourierCoeff_clustered(gpuComplex *in, uint_t N);
void createFourierCoeff_uniDistr(gpuComplex *in, uint_t N);
void createFourierCoeff_null(gpuComplex *in, uint_t N);
/** Example data: coefficients, then nodes x = drand48() - 0.5 (reference src/cuda_util.cpp:138-192). */
void getExampleData_clustered(cunfft_plan *plan);
void getExampleData_uniDistr(cunfft_plan *plan);
void getExampleDataAd_uniDistr(cunfft_plan *plan);
void getExampleData_null(cunfft_plan *plan);
void setExampleData(cunfft_plan *plan, gpuComplex *f, dTyp *x);
/** ||x - y||_inf (or ||x||_inf for y == NULL) and ||x-y||_inf / ||x||_inf
 *  (reference src/cuda_util.cpp:237-258). */
double l_infty(gpuComplex *x, gpuComplex *y, int n);
double compute_error_l_infty(gpuComplex *x, gpuComplex *y, int n);
/** Select device 0 and print its name.  Called by the reference's test driver
 *  (Tests/Scripts/simpleTest.cpp:379) but defined nowhere in the reference. */
void findDevice(void);

#ifdef __cplusplus
}
#endif

#define cudaVerify(x)                                                                  \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if (_e != cudaSuccess)                                                             \
      fprintf(stderr, "CUNFFT ERROR %s(%i): %s: %s\n", __FILE__, __LINE__, #x,         \
              cudaGetErrorString(_e));                                                 \
  } while (0)
#define cudaVerifyKernel(x)                                                            \
  do {                                                                                 \
    (x);                                                                               \
    cudaVerify(cudaGetLastError());                                                    \
  } while (0)
#define cufftVerify(x)                                                                 \
  do {                                                                                 \
    cufftResult _r = (x);                                                              \
    if (_r != CUFFT_SUCCESS)                                                           \
      fprintf(stderr, "CUNFFT ERROR %s(%i): %s: cuFFT error %d\n", __FILE__, __LINE__, \
              #x, (int)_r);                                                            \
  } while (0)
#define CHECK_LAUNCH_ERROR() cudaVerify(cudaGetLastError())

#endif /* CUNFFTUTIL_H_ */
