/*
 * cunfft.h -- drop-in C plan API of the GB300 NFFT library (libcunfft.so).
 *
 * Every declaration below replaces the reference function of the same name and
 * signature (reference src/cunfft.h, cited per entry).  Behaviour follows the
 * reference's call protocol:
 *   cunfft_init -> fill plan.x / plan.f_hat (or plan.f) on the host ->
 *   copyDataToDevice[Ad] -> cunfft_transform / cunfft_adjoint / cundft_* ->
 *   copyDataToHost[Ad] -> cunfft_finalize.
 * Transforms run on the GB300 kernels of this library and return when the
 * result is in plan.f_gpu (forward) or plan.fhat_gpu (adjoint), like the
 * reference's synchronous calls.
 *
 * Deviations, all deliberate:
 *   - errors never exit the process: each function records a status that
 *     cunfft_x_last_error(plan) returns and prints one line to stderr;
 *   - plans are independent: no global __constant__ state, so several plans
 *     (of any sizes) may be used in one process; one thread per plan;
 *   - cunfft_finalize does not call cudaDeviceReset (the reference's reset,
 *     src/cunfft.cu:409, destroys every other allocation in the process);
 *     resetDevice() still resets on request;
 *   - cunfft_reinitAd clears plan.f_hat and plan.g instead of allocating them
 *     again (the reference's re-allocation leaks, src/cunfft.cu:254-255);
 *   - CUNFFTTimes is always filled (the reference fills it only when built with
 *     MEASURED_TIMES).
 */
#ifndef CUNFFT1_H_
#define CUNFFT1_H_

#include "cunfft_typedefs.h"

#ifdef __cplusplus
extern "C" {
#endif

/** Create and destroy a throw-away 1D cuFFT plan (reference src/cunfft.h:35). */
void warmUp_createPlan(uint_t *n);

/** Upload f_hat and x (reference src/cunfft.h:47). */
void copyDataToDevice(cunfft_plan *plan);
/** Upload f and x (reference src/cunfft.h:57). */
void copyDataToDeviceAd(cunfft_plan *plan);
/** Download f (reference src/cunfft.h:66). */
void copyDataToHost(cunfft_plan *plan);
/** Download f_hat (reference src/cunfft.h:75). */
void copyDataToHostAd(cunfft_plan *plan);
/** Download the device coefficients into arr (reference src/cunfft.h:83). */
void copy_f_hat_ToHost(cunfft_plan *plan, gpuComplex *arr);
/** Download the device samples into arr (reference src/cunfft.h:91). */
void copy_f_ToHost(cunfft_plan *plan, gpuComplex *arr);
/** Download the oversampled grid into plan.g (reference src/cunfft.h:98). */
void copy_g_ToHost(cunfft_plan *plan);
/** Download the device nodes into arr (reference src/cunfft.h:106). */
void copy_x_toHost(cunfft_plan *plan, dTyp *arr);

/** Forward NFFT f = A f_hat on the device arrays (reference src/cunfft.h:117). */
void cunfft_transform(cunfft_plan *plan);
/** Adjoint NFFT f_hat = A^H f on the device arrays (reference src/cunfft.h:124). */
void cunfft_adjoint(cunfft_plan *plan);
/** Create a Z2Z cuFFT plan of dimension dim and lengths n (reference src/cunfft.h:133). */
void cunfft_initPlan(int dim, uint_t *n, cufftHandle *h);
/** Destroy the plan's cuFFT handles (reference src/cunfft.h:139). */
void cunfft_freePlan(cunfft_plan *p);
/** Allocate and zero the device arrays (reference src/cunfft.h:145). */
void cunfft_initDevicePara(cunfft_plan *plan);
/** Plan with n_t = 2 next_pow2(N_t), m = CUT_OFF (reference src/cunfft.h:156). */
void cunfft_init(cunfft_plan *plan, int dim, uint_t *N, uint_t M_total);
/** Plan with caller-chosen n and flags (reference src/cunfft.h:168). */
void cunfft_initGuru(cunfft_plan *plan, int dim, uint_t *N, uint_t M_total, uint_t *n, unsigned flags);
/** Derived parameters, host/device allocation, cuFFT plans (reference src/cunfft.h:177). */
void cunfft_initHelp(cunfft_plan *plan);
/** Clear f, g and the device arrays before a new forward run (reference src/cunfft.h:185). */
void cunfft_reinit(cunfft_plan *plan);
/** Clear f_hat, g and the device arrays before a new adjoint run (reference src/cunfft.h:194). */
void cunfft_reinitAd(cunfft_plan *plan);
/** Free everything the plan owns (reference src/cunfft.h:200). */
void cunfft_finalize(cunfft_plan *plan);
/** Free the device arrays (reference src/cunfft.h:206). */
void cunfft_finalizeDevice(cunfft_plan *plan);
/** Zero the timers (reference src/cunfft.h:212). */
void resetCUNFFTTimes(NFFTTimeSpec *times);

/** Direct NDFT f = sum_k f_hat_k e^{-2 pi i k x} on the device (reference src/cunfft.h:222). */
void cundft_transform(cunfft_plan *plan);
/** Direct adjoint NDFT f_hat = sum_j f_j e^{+2 pi i k x_j} (reference src/cunfft.h:228). */
void cundft_adjoint(cunfft_plan *plan);

/** fg_exp_l[offset + l] = exp(-l^2/b), l < FILTER_SIZE (reference src/cunfft.h:242). */
void nfft_init_fg_exp_l(double *fg_exp_l, const double b, const int offset);

/** Fill a kdata record (reference src/cunfft.h:256). */
void setProperties(uint_t *N, uint_t *n, double *b, double *sigma, int dim, kdata *k_cpu);

/** cudaDeviceReset (reference src/cunfft.h:261). */
void resetDevice(void);

/** Status of the last call on this plan (0 = success; cunfft_x_status codes).
 *  No reference counterpart: the reference's functions return void and exit
 *  the process on errors in DEBUG builds. */
int cunfft_x_last_error(const cunfft_plan *plan);

/** Select the cut-off m for the next cunfft_init / cunfft_initGuru in this
 *  thread (1..15; default CUT_OFF).  No reference counterpart: the reference
 *  fixes m at compile time (src/config.h.in CUT_OFF). */
int cunfft_x_set_default_cutoff(int m);

#ifdef __cplusplus
}
#endif

#endif /* CUNFFT1_H_ */
