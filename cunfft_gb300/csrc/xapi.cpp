// xapi.cpp -- the cunfft_x_* extension API (include/cunfft_x.h) over the plan runtime.
#include <new>
#include <stdio.h>

#include "runtime.h"

struct cunfft_x_plan {
  cg::Plan p;
};

extern "C" {

int cunfft_x_plan_create(cunfft_x_plan** out, int d, const int64_t* N, const int64_t* n, int m, int precision,
                         int batch, void* stream) {
  if (!out || !N) return CUNFFT_X_INVALID_ARGUMENT;
  *out = nullptr;
  cunfft_x_plan* h = new (std::nothrow) cunfft_x_plan();
  if (!h) return CUNFFT_X_ALLOC_FAILED;
  int s = cg::plan_init(&h->p, d, N, n, m, precision, batch, (cudaStream_t)stream, nullptr);
  if (s != CUNFFT_X_SUCCESS) {
    fprintf(stderr, "cunfft_x_plan_create: %s\n", h->p.last_msg);
    cg::plan_release(&h->p);
    delete h;
    return s;
  }
  *out = h;
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_plan_destroy(cunfft_x_plan* h) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  cg::plan_release(&h->p);
  delete h;
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_set_nodes(cunfft_x_plan* h, const double* x, const int64_t* M_inst) {
  if (!h || !M_inst) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_set_nodes(&h->p, x, M_inst);
}

int cunfft_x_forward(cunfft_x_plan* h, const void* fhat, void* f) {
  if (!h || (!fhat && h->p.geo.Ntot) || (!f && h->p.M)) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_forward(&h->p, fhat, f);
}

int cunfft_x_adjoint(cunfft_x_plan* h, const void* f, void* fhat) {
  if (!h || (!fhat && h->p.geo.Ntot) || (!f && h->p.M)) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_adjoint(&h->p, f, fhat);
}

int cunfft_x_forward_graph(cunfft_x_plan* h, const void* fhat, void* f) {
  if (!h || (!fhat && h->p.geo.Ntot) || (!f && h->p.M)) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_run_graph(&h->p, 0, fhat, f);
}

int cunfft_x_adjoint_graph(cunfft_x_plan* h, const void* f, void* fhat) {
  if (!h || (!fhat && h->p.geo.Ntot) || (!f && h->p.M)) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_run_graph(&h->p, 1, f, fhat);
}

int cunfft_x_ndft_forward(cunfft_x_plan* h, const void* fhat, void* f) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_ndft_forward(&h->p, fhat, f);
}

int cunfft_x_ndft_adjoint(cunfft_x_plan* h, const void* f, void* fhat) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_ndft_adjoint(&h->p, f, fhat);
}

int cunfft_x_ndft_adjoint_at(cunfft_x_plan* h, const void* f, const int64_t* kidx, int64_t nsel, void* out) {
  if (!h || (!kidx && nsel)) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_ndft_adjoint(&h->p, f, out, kidx, nsel);
}

int cunfft_x_node_gradient(cunfft_x_plan* h, const void* fhat, const void* grad_f, double* grad_x) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_node_gradient(&h->p, fhat, grad_f, grad_x);
}

int cunfft_x_interp(cunfft_x_plan* h, const void* g, void* f) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_interp_only(&h->p, g, f);
}

int cunfft_x_spread(cunfft_x_plan* h, const void* f, void* g) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_spread_only(&h->p, f, g);
}

int cunfft_x_set_stream(cunfft_x_plan* h, void* stream) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  cg::Plan& p = h->p;
  if (p.own_stream && p.stream && p.stream != (cudaStream_t)stream) {
    cudaStreamSynchronize(p.stream);
    cudaStreamDestroy(p.stream);
    p.own_stream = false;
  }
  if (stream) {
    p.stream = (cudaStream_t)stream;
  } else if (!p.own_stream) {
    if (cudaStreamCreate(&p.stream) != cudaSuccess) return CUNFFT_X_CUDA_ERROR;
    p.own_stream = true;
  }
  return CUNFFT_X_SUCCESS;
}

void* cunfft_x_get_stream(const cunfft_x_plan* h) { return h ? (void*)h->p.stream : nullptr; }

int cunfft_x_set_tiling(cunfft_x_plan* h, const int* T, int chunk) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  h->p.chunk_override = chunk > 0 ? chunk : 0;
  int s = cg::plan_choose_tiling(&h->p, T, chunk);
  if (s != CUNFFT_X_SUCCESS) return s;
  return CUNFFT_X_SUCCESS;  // re-binned lazily by the next transform
}

int cunfft_x_autotune(cunfft_x_plan* h, int reps) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_autotune(&h->p, reps);
}

int cunfft_x_get_tiling(const cunfft_x_plan* h, int* T, int* chunk, int* threads) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  if (T)
    for (int t = 0; t < 3; ++t) T[t] = h->p.tl.T[t];
  if (chunk) *chunk = h->p.tl.chunk;
  if (threads) *threads = h->p.tl.threads;
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_set_spread_kernel(cunfft_x_plan* h, int kind) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_set_spread_kernel(&h->p, kind);
}

int cunfft_x_get_spread_kernel(const cunfft_x_plan* h, int* kind) {
  if (!h || !kind) return CUNFFT_X_INVALID_ARGUMENT;
  *kind = cg::plan_spread_kernel(&h->p);
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_set_window(cunfft_x_plan* h, int window) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_set_window(&h->p, window);
}

int cunfft_x_get_window(const cunfft_x_plan* h, int* window) {
  if (!h || !window) return CUNFFT_X_INVALID_ARGUMENT;
  *window = cg::plan_window(&h->p);
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_forward_host(cunfft_x_plan* h, const double* x_host, const int64_t* M, const void* fhat_host,
                          void* f_host) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_forward_host(&h->p, x_host, M, fhat_host, f_host);
}

int cunfft_x_adjoint_host(cunfft_x_plan* h, const void* f_host, void* fhat_host) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_adjoint_host(&h->p, f_host, fhat_host);
}

int cunfft_x_set_interp_kernel(cunfft_x_plan* h, int kind) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  return cg::plan_set_interp_kernel(&h->p, kind);
}

int cunfft_x_get_interp_kernel(const cunfft_x_plan* h, int* kind) {
  if (!h || !kind) return CUNFFT_X_INVALID_ARGUMENT;
  *kind = cg::plan_interp_kernel(&h->p);
  return CUNFFT_X_SUCCESS;
}

static double ev_seconds(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.0;
  }
  return ms * 1e-3;
}

int cunfft_x_stage_times(cunfft_x_plan* h, double* t_bin, double* t_roc, double* t_fft, double* t_conv) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  cg::Plan& p = h->p;
  if (cudaStreamSynchronize(p.stream) != cudaSuccess) return CUNFFT_X_CUDA_ERROR;
  // forward records 0 roc 1 fft 2 conv 3; adjoint records 0 conv 1 fft 2 roc 3 (the
  // reference's adjoint runs gridding, FFT, roll-off: src/cunfft.cu:209-224)
  const double s01 = ev_seconds(p.ev[0], p.ev[1]), s12 = ev_seconds(p.ev[1], p.ev[2]),
               s23 = ev_seconds(p.ev[2], p.ev[3]);
  const bool adj = p.last_dir == 1;
  if (t_bin) *t_bin = ev_seconds(p.ev[6], p.ev[7]);
  if (t_fft) *t_fft = s12;
  if (t_roc) *t_roc = adj ? s23 : s01;
  if (t_conv) *t_conv = adj ? s01 : s23;
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_synchronize(cunfft_x_plan* h) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  cg::Plan& p = h->p;
  cudaError_t e = cudaStreamSynchronize(p.stream);
  if (e != cudaSuccess) return cg::check_cuda(&p, e, "cudaStreamSynchronize");
  CG_TRY(cg::plan_host_path_sync(&p));
  // device-side status: a bounded wait in a kernel that gave up (the flag is cleared on read)
  int32_t flag = 0;
  if (p.bins.status) {
    e = cudaMemcpyAsync(&flag, p.bins.status, sizeof(flag), cudaMemcpyDeviceToHost, p.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p.stream);
    if (e != cudaSuccess) return cg::check_cuda(&p, e, "read device status");
    if (flag != 0) {
      cudaMemsetAsync(p.bins.status, 0, sizeof(int32_t), p.stream);
      return cg::set_status(&p, CUNFFT_X_DEVICE_CHECK_FAILED,
                            "device check failed (code %d): a tensor-core completion wait gave up", (int)flag);
    }
  }
  return CUNFFT_X_SUCCESS;
}

int cunfft_x_check_wait_timeout(cunfft_x_plan* h) {
  if (!h) return CUNFFT_X_INVALID_ARGUMENT;
  cg::Plan& p = h->p;
  if (!p.bins.status) return CUNFFT_X_INVALID_ARGUMENT;
  const cudaError_t e = cg::launch_wait_gives_up(p.bins.status, p.stream);
  return e == cudaSuccess ? CUNFFT_X_SUCCESS : cg::check_cuda(&p, e, "k_wait_gives_up launch");
}

const char* cunfft_x_last_message(const cunfft_x_plan* h) { return h ? h->p.last_msg : ""; }

const char* cunfft_x_status_string(int s) {
  switch (s) {
    case CUNFFT_X_SUCCESS: return "success";
    case CUNFFT_X_INVALID_ARGUMENT: return "invalid argument";
    case CUNFFT_X_ALLOC_FAILED: return "allocation failed";
    case CUNFFT_X_CUFFT_ERROR: return "cuFFT error";
    case CUNFFT_X_CUDA_ERROR: return "CUDA error";
    case CUNFFT_X_NODES_NOT_SET: return "nodes not set";
    case CUNFFT_X_UNSUPPORTED: return "unsupported";
    case CUNFFT_X_DEVICE_CHECK_FAILED: return "device-side check failed";
    default: return "unknown status";
  }
}

void* cunfft_x_grid(const cunfft_x_plan* h) { return h ? h->p.g : nullptr; }

const char* cunfft_x_version(void) { return "cunfft-gb300 0.1 (sm_103a)"; }

}  // extern "C"
