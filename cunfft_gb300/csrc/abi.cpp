// abi.cpp -- the drop-in C plan API (include/cunfft.h) over the GB300 plan runtime.
//
// Each function mirrors the reference function of the same name (reference
// src/cunfft.cu:60-444, src/cunfft_wrapper.cu:252-286): same arguments, same
// plan members read and written, same host/device copy semantics.  The GB300
// runtime state of a cunfft_plan (binning buffers, roll-off tables, stream,
// events) lives in a side table keyed by the plan's address.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <unordered_map>

#include "cunfft.h"
#include "runtime.h"

namespace {

struct AbiState {
  cg::Plan p;
  bool device_ready = false;
};

std::mutex g_mu;
std::unordered_map<const cunfft_plan*, AbiState*> g_plans;
thread_local int t_default_m = CUT_OFF;

AbiState* state_of(const cunfft_plan* plan) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_plans.find(plan);
  return it == g_plans.end() ? nullptr : it->second;
}

AbiState* ensure_state(cunfft_plan* plan) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_plans.find(plan);
  if (it != g_plans.end()) return it->second;
  AbiState* s = new AbiState();
  g_plans[plan] = s;
  return s;
}

void drop_state(const cunfft_plan* plan) {
  AbiState* s = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_plans.find(plan);
    if (it == g_plans.end()) return;
    s = it->second;
    g_plans.erase(it);
  }
  cg::plan_release(&s->p);
  delete s;
}

// Errors never exit: record the status on the plan's state and print one line.
int report(AbiState* s, int code, const char* where) {
  if (code != CUNFFT_X_SUCCESS) {
    if (s) fprintf(stderr, "CUNFFT ERROR %s: %s\n", where, s->p.last_msg[0] ? s->p.last_msg : cunfft_x_status_string(code));
    else fprintf(stderr, "CUNFFT ERROR %s: %s\n", where, cunfft_x_status_string(code));
  }
  return code;
}

int cuda_call(AbiState* s, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return CUNFFT_X_SUCCESS;
  int code = s ? cg::check_cuda(&s->p, e, where) : CUNFFT_X_CUDA_ERROR;
  if (!s) fprintf(stderr, "CUNFFT ERROR %s: %s\n", where, cudaGetErrorString(e));
  else report(s, code, where);
  return code;
}

double seconds_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.0;
  }
  return ms * 1e-3;
}

int64_t next_pow2(int64_t v) {
  int64_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

// Binds the plan's device arrays to its runtime state (creates it if needed).
int bind_runtime(cunfft_plan* plan, AbiState* s) {
  if (s->device_ready) return CUNFFT_X_SUCCESS;
  int64_t N[3] = {1, 1, 1}, n[3] = {1, 1, 1};
  for (int t = 0; t < plan->d; ++t) {
    N[t] = plan->N[t];
    n[t] = plan->n[t];
  }
  int st = cg::plan_init(&s->p, plan->d, N, n, plan->m, cg::kF64, 1, nullptr, plan->g_gpu);
  if (st != CUNFFT_X_SUCCESS) return report(s, st, "cunfft_initHelp");
  s->device_ready = true;
  return CUNFFT_X_SUCCESS;
}

void fill_fg(cunfft_plan* plan) {
  const int W = 2 * plan->m + 2;
  free(plan->fg_exp_l_cpu);
  plan->fg_exp_l_cpu = (double*)calloc((size_t)W * MAX_DIM, sizeof(double));
  for (int t = 0; t < plan->d; ++t) {
    // exp(-l^2/b) by the recurrence of reference src/cunfft.cu:60-76
    double b0 = exp(-1.0 / plan->b[t]), b0sq = b0 * b0, b1 = 1.0, b2;
    double* out = plan->fg_exp_l_cpu + t * W;
    out[0] = 1.0;
    for (int l = 1; l < W; ++l) {
      b2 = b1 * b0;
      b1 *= b0sq;
      out[l] = out[l - 1] * b2;
    }
  }
}

int alloc_device(cunfft_plan* plan, AbiState* s) {
  if (cuda_call(s, cg::plan_malloc((void**)&plan->g_gpu, sizeof(gpuComplex) * plan->n_total), "cudaMalloc g")) return s->p.last_status;
  if (cuda_call(s, cudaMemset(plan->g_gpu, 0, sizeof(gpuComplex) * plan->n_total), "cudaMemset g")) return s->p.last_status;
  if (cuda_call(s, cg::plan_malloc((void**)&plan->fhat_gpu, sizeof(gpuComplex) * plan->N_total), "cudaMalloc f_hat")) return s->p.last_status;
  if (cuda_call(s, cudaMemset(plan->fhat_gpu, 0, sizeof(gpuComplex) * plan->N_total), "cudaMemset f_hat")) return s->p.last_status;
  if (cuda_call(s, cg::plan_malloc((void**)&plan->x_gpu, sizeof(dTyp) * plan->M_total * plan->d + 8), "cudaMalloc x")) return s->p.last_status;
  if (cuda_call(s, cudaMemset(plan->x_gpu, 0, sizeof(dTyp) * plan->M_total * plan->d + 8), "cudaMemset x")) return s->p.last_status;
  if (cuda_call(s, cg::plan_malloc((void**)&plan->f_gpu, sizeof(gpuComplex) * plan->M_total + 16), "cudaMalloc f")) return s->p.last_status;
  if (cuda_call(s, cudaMemset(plan->f_gpu, 0, sizeof(gpuComplex) * plan->M_total + 16), "cudaMemset f")) return s->p.last_status;
  return CUNFFT_X_SUCCESS;
}

void free_device(cunfft_plan* plan) {
  cudaFree(plan->x_gpu);
  cudaFree(plan->f_gpu);
  cudaFree(plan->fhat_gpu);
  cudaFree(plan->g_gpu);
  plan->x_gpu = nullptr;
  plan->f_gpu = nullptr;
  plan->fhat_gpu = nullptr;
  plan->g_gpu = nullptr;
}

}  // namespace

extern "C" {

int cunfft_x_last_error(const cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  return s ? s->p.last_status : CUNFFT_X_INVALID_ARGUMENT;
}

int cunfft_x_set_default_cutoff(int m) {
  if (m < 1 || m > 15) return CUNFFT_X_INVALID_ARGUMENT;
  t_default_m = m;
  return CUNFFT_X_SUCCESS;
}

void nfft_init_fg_exp_l(double* fg_exp_l, const double b, const int offset) {
  double b0 = exp(-1.0 / b), b0sq = b0 * b0, b1 = 1.0, b2;
  fg_exp_l[offset] = 1.0;
  for (int l = 1; l < FILTER_SIZE; ++l) {
    b2 = b1 * b0;
    b1 *= b0sq;
    fg_exp_l[l + offset] = fg_exp_l[l - 1 + offset] * b2;
  }
}

void setProperties(uint_t* N, uint_t* n, double* b, double* sigma, int dim, kdata* k) {
  for (int i = 0; i < dim; ++i) {
    k->N[i] = N[i];
    k->n[i] = n[i];
    k->b[i] = b[i];
    k->bsqrt[i] = sqrt(b[i]);
    k->fac[i] = (M_PI * M_PI * b[i]) / (double)(n[i] * n[i]);
    k->sigma[i] = sigma[i];
  }
}

void warmUp_createPlan(uint_t* n) {
  cufftHandle h;
  if (cufftPlan1d(&h, (int)n[0], CUFFT_Z2Z, 1) == CUFFT_SUCCESS) cufftDestroy(h);
  else fprintf(stderr, "CUNFFT ERROR warmUp_createPlan: cufftPlan1d failed\n");
  cudaDeviceSynchronize();
}

void resetCUNFFTTimes(NFFTTimeSpec* t) {
  t->runTime = 0.0;
  t->time_CONV = 0.0;
  t->time_COPY_IN = 0.0;
  t->time_COPY_OUT = 0.0;
  t->time_FFT = 0.0;
  t->time_ROC = 0.0;
}

void cunfft_initPlan(int dim, uint_t* n, cufftHandle* h) {
  cufftResult r;
  if (dim == 2) r = cufftPlan2d(h, (int)n[0], (int)n[1], CUFFT_Z2Z);
  else if (dim == 3) r = cufftPlan3d(h, (int)n[0], (int)n[1], (int)n[2], CUFFT_Z2Z);
  else r = cufftPlan1d(h, (int)n[0], CUFFT_Z2Z, 1);
  if (r != CUFFT_SUCCESS) {
    fprintf(stderr, "CUNFFT ERROR cunfft_initPlan: cuFFT error %d\n", (int)r);
    *h = 0;
  }
}

void cunfft_freePlan(cunfft_plan* p) {
  if (p->fft_backward) cufftDestroy(p->fft_backward);
  if (p->fft_forward) cufftDestroy(p->fft_forward);
  p->fft_backward = 0;
  p->fft_forward = 0;
  AbiState* s = state_of(p);
  if (s) {
    s->p.fft_fwd_ext = 0;
    s->p.fft_bwd_ext = 0;
  }
}

void cunfft_initDevicePara(cunfft_plan* plan) {
  AbiState* s = ensure_state(plan);
  if (alloc_device(plan, s) != CUNFFT_X_SUCCESS) return;
  // the runtime borrows g_gpu as its oversampled grid
  if (s->device_ready) s->p.g = plan->g_gpu;
}

void cunfft_init(cunfft_plan* plan, int dim, uint_t* N, uint_t M_total) {
  plan->d = dim;
  plan->N = (uint_t*)malloc(sizeof(uint_t) * dim);
  plan->n = (uint_t*)malloc(sizeof(uint_t) * dim);
  for (int t = 0; t < dim; ++t) {
    plan->N[t] = N[t];
    plan->n[t] = 2 * next_pow2(N[t]);
  }
  plan->M_total = M_total;
  plan->m = t_default_m;
  plan->flags = CUFFT_INIT | CUFFT_BOTH;
  cunfft_initHelp(plan);
}

void cunfft_initGuru(cunfft_plan* plan, int dim, uint_t* N, uint_t M_total, uint_t* n, unsigned flags) {
  plan->d = dim;
  plan->N = (uint_t*)malloc(sizeof(uint_t) * dim);
  plan->n = (uint_t*)malloc(sizeof(uint_t) * dim);
  for (int t = 0; t < dim; ++t) {
    plan->N[t] = N[t];
    plan->n[t] = n[t];
  }
  plan->M_total = M_total;
  plan->m = t_default_m;
  plan->flags = flags;
  cunfft_initHelp(plan);
}

void cunfft_initHelp(cunfft_plan* plan) {
  AbiState* s = ensure_state(plan);
  s->device_ready = false;
  plan->N_total = 1;
  plan->n_total = 1;
  for (int t = 0; t < plan->d; ++t) {
    plan->N_total *= plan->N[t];
    plan->n_total *= plan->n[t];
  }
  plan->sigma = (double*)malloc(sizeof(double) * plan->d);
  plan->b = (double*)malloc(sizeof(double) * plan->d);
  for (int t = 0; t < plan->d; ++t) {
    plan->sigma[t] = (double)plan->n[t] / (double)plan->N[t];
    plan->b[t] = (2.0 * plan->sigma[t]) / (2.0 * plan->sigma[t] - 1.0) * ((double)plan->m / M_PI);
  }
  plan->fg_exp_l_cpu = nullptr;
  fill_fg(plan);
  plan->g_hat = nullptr;
  resetCUNFFTTimes(&plan->CUNFFTTimes);
  plan->CUNFFTTimes.time_else = 0.0;
  plan->x = nullptr; plan->f_hat = nullptr; plan->f = nullptr; plan->g = nullptr;
  if (cuda_call(s, cudaMallocHost((void**)&plan->x, sizeof(dTyp) * plan->M_total * plan->d + 8), "cudaMallocHost x")) return;
  if (cuda_call(s, cudaMallocHost((void**)&plan->f_hat, sizeof(gpuComplex) * plan->N_total), "cudaMallocHost f_hat")) return;
  if (cuda_call(s, cudaMallocHost((void**)&plan->f, sizeof(gpuComplex) * plan->M_total + 16), "cudaMallocHost f")) return;
  if (cuda_call(s, cudaMallocHost((void**)&plan->g, sizeof(gpuComplex) * plan->n_total), "cudaMallocHost g")) return;
  memset(plan->x, 0, sizeof(dTyp) * plan->M_total * plan->d);
  memset(plan->f_hat, 0, sizeof(gpuComplex) * plan->N_total);
  memset(plan->f, 0, sizeof(gpuComplex) * plan->M_total);
  memset(plan->g, 0, sizeof(gpuComplex) * plan->n_total);
  plan->fft_backward = 0;
  plan->fft_forward = 0;
  plan->g_gpu = nullptr; plan->fhat_gpu = nullptr; plan->x_gpu = nullptr; plan->f_gpu = nullptr;
  if (alloc_device(plan, s) != CUNFFT_X_SUCCESS) return;
  if (bind_runtime(plan, s) != CUNFFT_X_SUCCESS) return;
  if (plan->flags & CUFFT_INIT) {
    if (plan->flags & CUFFT_BOTH) {
      cunfft_initPlan(plan->d, plan->n, &plan->fft_forward);
      cunfft_initPlan(plan->d, plan->n, &plan->fft_backward);
    }
    if (plan->flags & CUFFT_FORW) cunfft_initPlan(plan->d, plan->n, &plan->fft_forward);
    if (plan->flags & CUFFT_BACKW) cunfft_initPlan(plan->d, plan->n, &plan->fft_backward);
  }
  cg::set_status(&s->p, CUNFFT_X_SUCCESS, nullptr);
}

static int upload(cunfft_plan* plan, AbiState* s, bool adjoint) {
  cg::Plan& p = s->p;
  cudaEvent_t a = p.ev[4], b = p.ev[5];
  cudaEventRecord(a, 0);
  if (!adjoint) {
    if (cuda_call(s, cudaMemcpy(plan->fhat_gpu, plan->f_hat, sizeof(gpuComplex) * plan->N_total, cudaMemcpyHostToDevice),
                  "copyDataToDevice f_hat"))
      return p.last_status;
  } else {
    if (cuda_call(s, cudaMemcpy(plan->f_gpu, plan->f, sizeof(gpuComplex) * plan->M_total, cudaMemcpyHostToDevice),
                  "copyDataToDeviceAd f"))
      return p.last_status;
  }
  if (cuda_call(s, cudaMemcpy(plan->x_gpu, plan->x, sizeof(dTyp) * plan->M_total * plan->d, cudaMemcpyHostToDevice),
                "copyDataToDevice x"))
    return p.last_status;
  cudaEventRecord(b, 0);
  cudaEventSynchronize(b);
  plan->CUNFFTTimes.time_COPY_IN = seconds_between(a, b);
  return CUNFFT_X_SUCCESS;
}

void copyDataToDevice(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (!s) return (void)report(nullptr, CUNFFT_X_INVALID_ARGUMENT, "copyDataToDevice: plan not initialised");
  upload(plan, s, false);
}

void copyDataToDeviceAd(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (!s) return (void)report(nullptr, CUNFFT_X_INVALID_ARGUMENT, "copyDataToDeviceAd: plan not initialised");
  upload(plan, s, true);
}

static void download(AbiState* s, void* dst, const void* src, size_t bytes, double* t_out, const char* where) {
  cudaEvent_t a = s ? s->p.ev[4] : nullptr, b = s ? s->p.ev[5] : nullptr;
  if (a) cudaEventRecord(a, 0);
  if (cuda_call(s, cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), where)) return;
  if (b) {
    cudaEventRecord(b, 0);
    cudaEventSynchronize(b);
    if (t_out) *t_out = seconds_between(a, b);
  }
}

void copyDataToHost(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  download(s, plan->f, plan->f_gpu, sizeof(gpuComplex) * plan->M_total, &plan->CUNFFTTimes.time_COPY_OUT,
           "copyDataToHost");
}

void copyDataToHostAd(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  download(s, plan->f_hat, plan->fhat_gpu, sizeof(gpuComplex) * plan->N_total, &plan->CUNFFTTimes.time_COPY_OUT,
           "copyDataToHostAd");
}

void copy_f_ToHost(cunfft_plan* plan, gpuComplex* arr) {
  download(state_of(plan), arr, plan->f_gpu, sizeof(gpuComplex) * plan->M_total, nullptr, "copy_f_ToHost");
}

void copy_g_ToHost(cunfft_plan* plan) {
  download(state_of(plan), plan->g, plan->g_gpu, sizeof(gpuComplex) * plan->n_total, nullptr, "copy_g_ToHost");
}

void copy_f_hat_ToHost(cunfft_plan* plan, gpuComplex* arr) {
  download(state_of(plan), arr, plan->fhat_gpu, sizeof(gpuComplex) * plan->N_total, nullptr, "copy_f_hat_ToHost");
}

void copy_x_toHost(cunfft_plan* plan, dTyp* arr) {
  download(state_of(plan), arr, plan->x_gpu, sizeof(dTyp) * plan->M_total * plan->d, nullptr, "copy_x_toHost");
}

// The transform binds the current device nodes every call (plan.x_gpu may have
// been rewritten by the caller since the last one) and returns when the result
// is in device memory, like the reference's synchronous stages.
static int prepare(cunfft_plan* plan, AbiState* s, const char* where) {
  if (!s) return report(nullptr, CUNFFT_X_INVALID_ARGUMENT, where);
  if (bind_runtime(plan, s) != CUNFFT_X_SUCCESS) return s->p.last_status;
  cg::Plan& p = s->p;
  p.g = plan->g_gpu;
  p.fft_fwd_ext = plan->fft_forward;
  p.fft_bwd_ext = plan->fft_backward;
  int64_t M = plan->M_total;
  int st = cg::plan_set_nodes(&p, plan->x_gpu, &M);
  return report(s, st, where);
}

static void finish(cunfft_plan* plan, AbiState* s, bool adjoint, const char* where) {
  cg::Plan& p = s->p;
  cudaError_t e = cudaStreamSynchronize(p.stream);
  if (e != cudaSuccess) {
    report(s, cg::check_cuda(&p, e, where), where);
    return;
  }
  const double t01 = seconds_between(p.ev[0], p.ev[1]), t12 = seconds_between(p.ev[1], p.ev[2]),
               t23 = seconds_between(p.ev[2], p.ev[3]), tb = seconds_between(p.ev[6], p.ev[7]);
  plan->CUNFFTTimes.time_FFT = t12;
  if (!adjoint) {
    plan->CUNFFTTimes.time_ROC = t01;
    plan->CUNFFTTimes.time_CONV = t23 + tb;
  } else {
    plan->CUNFFTTimes.time_CONV = t01 + tb;
    plan->CUNFFTTimes.time_ROC = t23;
  }
}

void cunfft_transform(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (prepare(plan, s, "cunfft_transform") != CUNFFT_X_SUCCESS) return;
  int st = cg::plan_forward(&s->p, plan->fhat_gpu, plan->f_gpu);
  if (report(s, st, "cunfft_transform") != CUNFFT_X_SUCCESS) return;
  finish(plan, s, false, "cunfft_transform");
}

void cunfft_adjoint(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (prepare(plan, s, "cunfft_adjoint") != CUNFFT_X_SUCCESS) return;
  int st = cg::plan_adjoint(&s->p, plan->f_gpu, plan->fhat_gpu);
  if (report(s, st, "cunfft_adjoint") != CUNFFT_X_SUCCESS) return;
  finish(plan, s, true, "cunfft_adjoint");
}

void cundft_transform(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (prepare(plan, s, "cundft_transform") != CUNFFT_X_SUCCESS) return;
  int st = cg::plan_ndft_forward(&s->p, plan->fhat_gpu, plan->f_gpu);
  if (report(s, st, "cundft_transform") != CUNFFT_X_SUCCESS) return;
  cudaError_t e = cudaStreamSynchronize(s->p.stream);
  if (e != cudaSuccess) report(s, cg::check_cuda(&s->p, e, "cundft_transform"), "cundft_transform");
}

void cundft_adjoint(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (prepare(plan, s, "cundft_adjoint") != CUNFFT_X_SUCCESS) return;
  int st = cg::plan_ndft_adjoint(&s->p, plan->f_gpu, plan->fhat_gpu);
  if (report(s, st, "cundft_adjoint") != CUNFFT_X_SUCCESS) return;
  cudaError_t e = cudaStreamSynchronize(s->p.stream);
  if (e != cudaSuccess) report(s, cg::check_cuda(&s->p, e, "cundft_adjoint"), "cundft_adjoint");
}

void cunfft_reinit(cunfft_plan* plan) {
  AbiState* s = ensure_state(plan);
  resetCUNFFTTimes(&plan->CUNFFTTimes);
  if (s->device_ready) cudaStreamSynchronize(s->p.stream);
  free_device(plan);
  memset(plan->f, 0, sizeof(gpuComplex) * plan->M_total);
  memset(plan->g, 0, sizeof(gpuComplex) * plan->n_total);
  if (alloc_device(plan, s) != CUNFFT_X_SUCCESS) return;
  if (s->device_ready) s->p.g = plan->g_gpu;
  cudaDeviceSynchronize();
}

void cunfft_reinitAd(cunfft_plan* plan) {
  AbiState* s = ensure_state(plan);
  resetCUNFFTTimes(&plan->CUNFFTTimes);
  if (s->device_ready) cudaStreamSynchronize(s->p.stream);
  free_device(plan);
  memset(plan->f_hat, 0, sizeof(gpuComplex) * plan->N_total);
  memset(plan->g, 0, sizeof(gpuComplex) * plan->n_total);
  if (alloc_device(plan, s) != CUNFFT_X_SUCCESS) return;
  if (s->device_ready) s->p.g = plan->g_gpu;
  cudaDeviceSynchronize();
}

void cunfft_finalizeDevice(cunfft_plan* plan) {
  AbiState* s = state_of(plan);
  if (s && s->device_ready) cudaStreamSynchronize(s->p.stream);
  free_device(plan);
  cudaDeviceSynchronize();
}

void cunfft_finalize(cunfft_plan* plan) {
  if (plan->flags & CUFFT_INIT) cunfft_freePlan(plan);
  cudaFreeHost(plan->g);
  cudaFreeHost(plan->f);
  free(plan->fg_exp_l_cpu);
  cudaFreeHost(plan->x);
  cudaFreeHost(plan->f_hat);
  free(plan->sigma);
  free(plan->n);
  free(plan->N);
  free(plan->b);
  plan->g = nullptr; plan->f = nullptr; plan->fg_exp_l_cpu = nullptr; plan->x = nullptr; plan->f_hat = nullptr;
  plan->sigma = nullptr; plan->n = nullptr; plan->N = nullptr; plan->b = nullptr;
  cunfft_finalizeDevice(plan);
  drop_state(plan);
}

void resetDevice(void) { cudaDeviceReset(); }

}  // extern "C"
