// hostpath.cpp -- forward and adjoint transforms from pinned host memory with the
// host<->device copies on two copy streams (uploads, downloads) that run beside
// the plan stream's kernels.
//
// The reference copies synchronously before and after every transform
// (copyDataToDevice / copyDataToHost, src/cunfft.cu:107-190).  Here a forward
// call uploads the nodes first (the binning waits for them), then the coefficients
// (overlapping the binning); its samples download while the plan stream already
// runs the next call's work.  An adjoint call's upload can start during the
// preceding forward.  Plan-owned device staging buffers are reused across calls;
// events order every reuse (a buffer is rewritten only after the work that reads
// it has completed).  All of it is asynchronous with respect to the host:
// cunfft_x_synchronize waits for the plan stream and both copy streams.
#include <algorithm>

#include "runtime.h"

namespace cg {

struct HostPath {
  cudaStream_t up = nullptr, down = nullptr;
  // Recorded on the plan stream: x_free[b] when every kernel enqueued before the
  // switch away from node buffer b has run (the binning, and any re-binning, NDFT
  // or gradient that read those nodes), forward done (coefficient staging free,
  // samples ready), adjoint done (sample staging free, coefficients ready).  On the
  // copy streams: uploads landed, downloads done.
  cudaEvent_t x_free[2] = {nullptr, nullptr}, fwd_done = nullptr, adj_done = nullptr;
  cudaEvent_t x_in = nullptr, fh_in = nullptr, f_in = nullptr, f_out_done = nullptr, fh_out_done = nullptr;
  double* x[2] = {nullptr, nullptr};  // [cap_M * d] each, alternating between node uploads
  int xb = 1;                         // buffer of the latest upload
  void* fh_in_dev = nullptr;   // [batch N_total] coefficients in
  void* fh_out_dev = nullptr;  // [batch N_total] coefficients out
  void* f_in_dev = nullptr;    // [cap_M] samples in
  void* f_out_dev = nullptr;   // [cap_M] samples out
  int64_t cap_M = -1;
};

static int host_path(Plan* p, HostPath** out) {
  if (p->hp) {
    *out = p->hp;
    return CUNFFT_X_SUCCESS;
  }
  HostPath* h = new HostPath();
  p->hp = h;
  CG_TRY(check_cuda(p, cudaStreamCreateWithFlags(&h->up, cudaStreamNonBlocking), "cudaStreamCreate"));
  CG_TRY(check_cuda(p, cudaStreamCreateWithFlags(&h->down, cudaStreamNonBlocking), "cudaStreamCreate"));
  cudaEvent_t* evs[] = {&h->x_free[0], &h->x_free[1], &h->fwd_done,   &h->adj_done, &h->x_in,
                        &h->fh_in,     &h->f_in,      &h->f_out_done, &h->fh_out_done};
  for (cudaEvent_t* e : evs) CG_TRY(check_cuda(p, cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate"));
  const size_t coef = plan_elem_bytes(p) * (size_t)p->geo.Ntot * (size_t)p->geo.batch;
  CG_TRY(check_cuda(p, plan_malloc(&h->fh_in_dev, coef), "cudaMalloc host-path staging"));
  CG_TRY(check_cuda(p, plan_malloc(&h->fh_out_dev, coef), "cudaMalloc host-path staging"));
  *out = h;
  return CUNFFT_X_SUCCESS;
}

// Node staging for M nodes; growing it waits for every stream of the plan.
static int host_path_nodes(Plan* p, HostPath* h, int64_t M) {
  if (M <= h->cap_M) return CUNFFT_X_SUCCESS;
  CG_TRY(check_cuda(p, cudaStreamSynchronize(p->stream), "cudaStreamSynchronize"));
  CG_TRY(check_cuda(p, cudaStreamSynchronize(h->up), "cudaStreamSynchronize"));
  CG_TRY(check_cuda(p, cudaStreamSynchronize(h->down), "cudaStreamSynchronize"));
  if (p->x == h->x[0] || p->x == h->x[1]) p->nodes_set = false;  // bound nodes are about to be freed
  cudaFree(h->x[0]);
  cudaFree(h->x[1]);
  cudaFree(h->f_in_dev);
  cudaFree(h->f_out_dev);
  h->x[0] = h->x[1] = nullptr;
  h->f_in_dev = h->f_out_dev = nullptr;
  h->cap_M = -1;
  const int64_t cap = std::max<int64_t>(M, 1);
  for (int b = 0; b < 2; ++b)
    CG_TRY(check_cuda(p, plan_malloc(&h->x[b], sizeof(double) * (size_t)cap * p->geo.d), "cudaMalloc host-path staging"));
  CG_TRY(check_cuda(p, plan_malloc(&h->f_in_dev, plan_elem_bytes(p) * (size_t)cap), "cudaMalloc host-path staging"));
  CG_TRY(check_cuda(p, plan_malloc(&h->f_out_dev, plan_elem_bytes(p) * (size_t)cap), "cudaMalloc host-path staging"));
  h->cap_M = cap;
  return CUNFFT_X_SUCCESS;
}

int plan_forward_host(Plan* p, const double* x_host, const int64_t* M_inst, const void* fhat_host, void* f_host) {
  if (!fhat_host || !f_host) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "forward_host: NULL buffer");
  HostPath* h = nullptr;
  CG_TRY(host_path(p, &h));
  if (x_host) {
    if (!M_inst) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "forward_host: nodes given without counts");
    int64_t M = 0;
    for (int i = 0; i < p->geo.batch; ++i) M += M_inst[i] > 0 ? M_inst[i] : 0;
    CG_TRY(host_path_nodes(p, h, M));
    // switch node buffers: everything enqueued so far reads the current one at most
    const int b = h->xb ^ 1;
    CG_TRY(check_cuda(p, cudaEventRecord(h->x_free[h->xb], p->stream), "cudaEventRecord"));
    // buffer b is rewritten once every kernel enqueued before the previous switch has run
    CG_TRY(check_cuda(p, cudaStreamWaitEvent(h->up, h->x_free[b], 0), "cudaStreamWaitEvent"));
    CG_TRY(check_cuda(p, cudaMemcpyAsync(h->x[b], x_host, sizeof(double) * (size_t)M * p->geo.d, cudaMemcpyHostToDevice,
                                         h->up), "upload nodes"));
    CG_TRY(check_cuda(p, cudaEventRecord(h->x_in, h->up), "cudaEventRecord"));
    CG_TRY(check_cuda(p, cudaStreamWaitEvent(p->stream, h->x_in, 0), "cudaStreamWaitEvent"));
    h->xb = b;
    CG_TRY(plan_set_nodes(p, h->x[b], M_inst));
  } else if (!p->nodes_set) {
    return set_status(p, CUNFFT_X_NODES_NOT_SET, "forward_host: nodes not set");
  } else {
    CG_TRY(host_path_nodes(p, h, p->M));  // nodes bound elsewhere: sample staging for them
  }
  const size_t coef = plan_elem_bytes(p) * (size_t)p->geo.Ntot * (size_t)p->geo.batch;
  // coefficients: staging free once the previous forward is done; lands while the binning runs
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(h->up, h->fwd_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(check_cuda(p, cudaMemcpyAsync(h->fh_in_dev, fhat_host, coef, cudaMemcpyHostToDevice, h->up), "upload coefficients"));
  CG_TRY(check_cuda(p, cudaEventRecord(h->fh_in, h->up), "cudaEventRecord"));
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(p->stream, h->fh_in, 0), "cudaStreamWaitEvent"));
  // the sample staging is rewritten once the previous download has read it
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(p->stream, h->f_out_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(plan_forward(p, h->fh_in_dev, h->f_out_dev));
  CG_TRY(check_cuda(p, cudaEventRecord(h->fwd_done, p->stream), "cudaEventRecord"));
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(h->down, h->fwd_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(check_cuda(p, cudaMemcpyAsync(f_host, h->f_out_dev, plan_elem_bytes(p) * (size_t)p->M, cudaMemcpyDeviceToHost,
                                       h->down), "download samples"));
  CG_TRY(check_cuda(p, cudaEventRecord(h->f_out_done, h->down), "cudaEventRecord"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_adjoint_host(Plan* p, const void* f_host, void* fhat_host) {
  if (!f_host || !fhat_host) return set_status(p, CUNFFT_X_INVALID_ARGUMENT, "adjoint_host: NULL buffer");
  HostPath* h = nullptr;
  CG_TRY(host_path(p, &h));
  if (!p->nodes_set) return set_status(p, CUNFFT_X_NODES_NOT_SET, "adjoint_host: nodes not set");
  CG_TRY(host_path_nodes(p, h, p->M));
  // samples: staging free once the previous adjoint is done; lands while the plan stream works
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(h->up, h->adj_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(check_cuda(p, cudaMemcpyAsync(h->f_in_dev, f_host, plan_elem_bytes(p) * (size_t)p->M, cudaMemcpyHostToDevice, h->up),
                    "upload samples"));
  CG_TRY(check_cuda(p, cudaEventRecord(h->f_in, h->up), "cudaEventRecord"));
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(p->stream, h->f_in, 0), "cudaStreamWaitEvent"));
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(p->stream, h->fh_out_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(plan_adjoint(p, h->f_in_dev, h->fh_out_dev));
  CG_TRY(check_cuda(p, cudaEventRecord(h->adj_done, p->stream), "cudaEventRecord"));
  CG_TRY(check_cuda(p, cudaStreamWaitEvent(h->down, h->adj_done, 0), "cudaStreamWaitEvent"));
  CG_TRY(check_cuda(p, cudaMemcpyAsync(fhat_host, h->fh_out_dev, plan_elem_bytes(p) * (size_t)p->geo.Ntot * p->geo.batch,
                                       cudaMemcpyDeviceToHost, h->down), "download coefficients"));
  CG_TRY(check_cuda(p, cudaEventRecord(h->fh_out_done, h->down), "cudaEventRecord"));
  return set_status(p, CUNFFT_X_SUCCESS, nullptr);
}

int plan_host_path_sync(Plan* p) {
  if (!p->hp) return CUNFFT_X_SUCCESS;
  CG_TRY(check_cuda(p, cudaStreamSynchronize(p->hp->up), "cudaStreamSynchronize"));
  CG_TRY(check_cuda(p, cudaStreamSynchronize(p->hp->down), "cudaStreamSynchronize"));
  return CUNFFT_X_SUCCESS;
}

void plan_host_path_release(Plan* p) {
  HostPath* h = p->hp;
  if (!h) return;
  if (h->up) cudaStreamSynchronize(h->up);
  if (h->down) cudaStreamSynchronize(h->down);
  cudaEvent_t evs[] = {h->x_free[0], h->x_free[1], h->fwd_done, h->adj_done, h->x_in,
                       h->fh_in,     h->f_in,      h->f_out_done, h->fh_out_done};
  for (cudaEvent_t e : evs)
    if (e) cudaEventDestroy(e);
  if (h->up) cudaStreamDestroy(h->up);
  if (h->down) cudaStreamDestroy(h->down);
  cudaFree(h->x[0]);
  cudaFree(h->x[1]);
  cudaFree(h->fh_in_dev);
  cudaFree(h->fh_out_dev);
  cudaFree(h->f_in_dev);
  cudaFree(h->f_out_dev);
  delete h;
  p->hp = nullptr;
}

}  // namespace cg
