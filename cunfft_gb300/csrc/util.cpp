// util.cpp -- driver utilities of the plan API (include/cunfft_util.h).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cunfft_util.h"

extern "C" {

void showTimes(NFFTTimeSpec* t, int tfac) {
  const double f = tfac > 0 ? 1.0 / tfac : 1.0;
  printf("Runtime:\t %.2E s\n", t->runTime * f);
  printf("  ROC:\t\t %.2E s\n  FFT:\t\t %.2E s\n  CONV:\t\t %.2E s\n", t->time_ROC * f, t->time_FFT * f,
         t->time_CONV * f);
  printf("  COPY IN:\t %.2E s\n  COPY OUT:\t %.2E s\n", t->time_COPY_IN * f, t->time_COPY_OUT * f);
}

unsigned long getGPUMemProps_ToStdout(void) {
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
    cudaGetLastError();
    printf("# device memory: unavailable\n");
    return 0;
  }
  printf("# device memory: %.1f MB free of %.1f MB\n", free_b / 1048576.0, total_b / 1048576.0);
  return (unsigned long)free_b;
}

void showCPUMemUse(cunfft_plan* p) {
  const double bytes = sizeof(gpuComplex) * ((double)p->n_total + p->M_total + p->N_total) +
                       sizeof(dTyp) * (double)p->M_total * p->d;
  printf("# host memory used by the plan arrays: %.0f bytes (%.1f MB)\n", bytes, bytes / 1048576.0);
}

void showCoeff_double(const dTyp* x, int n, const char* text) {
  printf("\n %s\n", text);
  for (int k = 0; k < n; ++k) printf("%+.4e%s", x[k], (k % 4 == 3) ? "\n" : ", ");
  printf("\n");
}

void showCoeff_cuComplex(const gpuComplex* x, int n, const char* text) {
  printf("\n %s\n", text);
  for (int k = 0; k < n; ++k) printf("%+.4e %+.4ei%s", x[k].x, x[k].y, (k % 4 == 3) ? "\n" : ",  ");
  printf("\n");
}

uint_t prod_int(uint_t* vec, int d) {
  uint_t p = 1;
  for (int t = 0; t < d; ++t) p *= vec[t];
  return p;
}

uint_t next_power_of_2(uint_t N) {
  uint_t p = 1;
  while (p < N) p <<= 1;
  return p;
}

void createFourierCoeff_clustered(gpuComplex* in, uint_t N) {
  double kk = -(double)(N / 2);
  for (uint_t k = 0; k < N; ++k, kk += 1.0) {
    in[k].x = sin(10.0 * kk / (double)N) * exp(-pow(kk / pow((double)N, 0.8), 2));
    in[k].y = 0.0;
  }
}

void createFourierCoeff_uniDistr(gpuComplex* in, uint_t N) {
  for (uint_t k = 0; k < N; ++k) {
    in[k].x = drand48();
    in[k].y = drand48();
  }
}

void createFourierCoeff_null(gpuComplex* in, uint_t N) { memset(in, 0, sizeof(gpuComplex) * N); }

static void random_nodes(cunfft_plan* plan) {
  const uint_t M = plan->M_total * plan->d;
  for (uint_t i = 0; i < M; ++i) plan->x[i] = drand48() - 0.5;
}

void getExampleData_clustered(cunfft_plan* plan) {
  createFourierCoeff_clustered(plan->f_hat, plan->N_total);
  const uint_t M = plan->M_total * plan->d;
  double j = 0.0;
  for (uint_t i = 0; i < M; ++i, j += 1.0 / (double)M) plan->x[i] = pow(j, 1.0 / 100.0);
}

void getExampleData_uniDistr(cunfft_plan* plan) {
  createFourierCoeff_uniDistr(plan->f_hat, plan->N_total);
  random_nodes(plan);
}

void getExampleDataAd_uniDistr(cunfft_plan* plan) {
  createFourierCoeff_uniDistr(plan->f, plan->M_total);
  random_nodes(plan);
}

void getExampleData_null(cunfft_plan* plan) {
  createFourierCoeff_null(plan->f_hat, plan->N_total);
  random_nodes(plan);
}

void setExampleData(cunfft_plan* plan, gpuComplex* f, dTyp* x) {
  for (uint_t i = 0; i < plan->M_total * plan->d; ++i) plan->x[i] = x[i];
  for (uint_t i = 0; i < plan->M_total; ++i) plan->f[i] = f[i];
}

double l_infty(gpuComplex* x, gpuComplex* y, int n) {
  double r = 0.0;
  for (int k = 0; k < n; ++k) {
    const double v = y ? hypot(x[k].x - y[k].x, x[k].y - y[k].y) : hypot(x[k].x, x[k].y);
    if (v > r) r = v;
  }
  return r;
}

double compute_error_l_infty(gpuComplex* x, gpuComplex* y, int n) { return l_infty(x, y, n) / l_infty(x, NULL, n); }

void findDevice(void) {
  int dev = 0;
  cudaDeviceProp prop;
  if (cudaSetDevice(dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
    printf("# device %d: %s (cc %d.%d, %d SMs)\n", dev, prop.name, prop.major, prop.minor, prop.multiProcessorCount);
  else {
    cudaGetLastError();
    printf("# no CUDA device\n");
  }
}

}  // extern "C"
