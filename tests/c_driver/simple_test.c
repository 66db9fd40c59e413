/*
 * simple_test.c -- a C program that drives libcunfft.so through the reference's plan API
 * (include/cunfft.h, include/cunfft_util.h) the way the reference's test driver does
 * (Tests/Scripts/simpleTest.cpp:62-177 forward, :179-260 adjoint): per repetition a fresh
 * plan, example data from drand48, the direct transform on the device, reinit, the fast
 * transform, and the relative l_inf error between the two.  The reference's logged error
 * tables come from ten such repetitions in one process; the tenth repetition's error is
 * a known answer of the method (the drand48 stream runs on across repetitions).
 *
 * Usage: simple_test <fwd|adj> <reps> <d> <N_0> [<N_1> [<N_2>]]   (M = N_total)
 * Prints one line per repetition: "rep <r> e_inf <value> status <code>".
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cunfft.h"
#include "cunfft_util.h"

static double run_forward(uint_t *N, uint_t M, int d, int *status) {
  cunfft_plan p;
  cunfft_init(&p, d, N, M);
  if ((*status = cunfft_x_last_error(&p)) != 0) { /* no device or no memory: the plan holds no arrays */
    cunfft_finalize(&p);
    return -1.0;
  }
  getExampleData_uniDistr(&p);
  copyDataToDevice(&p);
  gpuComplex *cundft = (gpuComplex *)malloc(sizeof(gpuComplex) * (size_t)p.M_total);
  cundft_transform(&p);
  copy_f_ToHost(&p, cundft);
  cunfft_reinit(&p);
  copyDataToDevice(&p);
  cunfft_transform(&p);
  copyDataToHost(&p);
  const double err = compute_error_l_infty(cundft, p.f, (int)p.M_total);
  *status = cunfft_x_last_error(&p);
  free(cundft);
  cunfft_finalize(&p);
  return err;
}

static double run_adjoint(uint_t *N, uint_t M, int d, int *status) {
  cunfft_plan p;
  cunfft_init(&p, d, N, M);
  if ((*status = cunfft_x_last_error(&p)) != 0) { /* no device or no memory: the plan holds no arrays */
    cunfft_finalize(&p);
    return -1.0;
  }
  getExampleDataAd_uniDistr(&p);
  copyDataToDeviceAd(&p);
  gpuComplex *cundft = (gpuComplex *)malloc(sizeof(gpuComplex) * (size_t)p.N_total);
  cundft_adjoint(&p);
  copy_f_hat_ToHost(&p, cundft);
  cunfft_reinitAd(&p);
  copyDataToDeviceAd(&p);
  cunfft_adjoint(&p);
  copyDataToHostAd(&p);
  const double err = compute_error_l_infty(cundft, p.f_hat, (int)p.N_total);
  *status = cunfft_x_last_error(&p);
  free(cundft);
  cunfft_finalize(&p);
  return err;
}

int main(int argc, char **argv) {
  if (argc < 5) {
    fprintf(stderr, "usage: %s <fwd|adj> <reps> <d> <N_0> [<N_1> [<N_2>]]\n", argv[0]);
    return 2;
  }
  const int adjoint = strcmp(argv[1], "adj") == 0;
  const int reps = atoi(argv[2]), d = atoi(argv[3]);
  if (d < 1 || d > 3 || argc != 4 + d || reps < 1) {
    fprintf(stderr, "bad arguments\n");
    return 2;
  }
  uint_t N[3] = {1, 1, 1}, M = 1;
  for (int t = 0; t < d; ++t) {
    N[t] = (uint_t)atol(argv[4 + t]);
    M *= N[t];
  }
  int failed = 0;
  for (int r = 0; r < reps; ++r) {
    int status = 0;
    const double e = adjoint ? run_adjoint(N, M, d, &status) : run_forward(N, M, d, &status);
    printf("rep %d e_inf %.6e status %d\n", r, e, status);
    failed |= status != 0;
  }
  return failed ? 1 : 0;
}
