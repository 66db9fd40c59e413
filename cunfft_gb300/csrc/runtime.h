// runtime.h -- host runtime of the GB300 NFFT: plan object, launchers, status codes.
//
// One Plan describes B transform instances that share d, N, n and m.  It owns the
// oversampled grid (unless the caller lends one, as the drop-in ABI does with
// cunfft_plan::g_gpu), the cuFFT plan, the binning buffers and a CUDA stream.
// Every kernel argument is passed by value: there is no global __constant__
// state, so any number of plans coexist and run concurrently on their streams.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include "common.cuh"
#include "cunfft_x.h"

namespace cg {

enum Precision { kF64 = CUNFFT_X_F64, kF32 = CUNFFT_X_F32 };

struct HostPath;  // copy streams and staging of the host-buffer transforms (hostpath.cpp)

struct Plan {
  Geom geo{};
  int prec = kF64;
  int num_sms = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  cufftHandle fft = 0;         // batched plan used for both directions
  bool own_fft = false;
  cufftHandle fft_fwd_ext = 0; // handles lent by the drop-in ABI (0: use fft)
  cufftHandle fft_bwd_ext = 0;
  void* g = nullptr;           // batch * ntot complex
  bool own_g = false;
  double* roc_tab = nullptr;   // per-dim roll-off factors 1 / phi_hat_t(k_t / n_t), sum_t N_t doubles
  Tiling tl{};
  Bins bins{};
  int64_t bins_capacity_M = -1;
  int64_t bins_capacity_tiles = -1;
  int64_t bins_capacity_keys = -1;  // sub-bin keys the bins hold room for (Tiling::sub_on)
  const double* x = nullptr;   // device nodes of the current node set
  int64_t M = 0;
  int64_t* M_inst = nullptr;   // host copy of per-instance node counts
  bool inst_off_current = false;  // bins.inst_off holds the offsets of M_inst
  bool nodes_set = false;
  int tile_override[kMaxDim] = {0, 0, 0};
  int chunk_override = 0;
  int spread_mode = CUNFFT_X_SPREAD_AUTO;  // requested spreading kernel
  int interp_mode = CUNFFT_X_INTERP_AUTO;  // requested interpolation kernel
  bool autotuned = false;
  int last_status = 0;
  char last_msg[256] = {0};
  // per-stage timing of the last call (seconds), recorded with events on the plan stream
  cudaEvent_t ev[8] = {};
  bool timing = false;
  int last_dir = 0;       // direction of the last timed transform: 0 forward, 1 adjoint
  double t_bin = 0, t_roc = 0, t_fft = 0, t_conv = 0;
  // CUDA graphs of the forward [0] and adjoint [1] stage sequences
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  const void* g_in[2] = {nullptr, nullptr};
  void* g_out[2] = {nullptr, nullptr};
  uint64_t g_gen[2] = {0, 0};
  uint64_t node_gen = 0;  // bumped by every node binding / tiling change
  HostPath* hp = nullptr; // created by the first host-buffer transform
  // tensor-core interpolation: the grid's padded FP16 hi/lo planes, their per-plane
  // inverse scales and their TMA map, created before its first launch (interp_tc_prepare)
  void* it_split = nullptr;
  float* it_pinv = nullptr;
  CUtensorMap it_tmap{};
  bool it_ready = false;
};

inline size_t plan_elem_bytes(const Plan* p) { return p->prec == kF64 ? 16 : 8; }

int plan_window(const Plan* p);
int plan_set_window(Plan* p, int window);

// return the status of a runtime call when it is not CUNFFT_X_SUCCESS
#define CG_TRY(expr)                          \
  do {                                        \
    int _s = (expr);                          \
    if (_s != CUNFFT_X_SUCCESS) return _s;    \
  } while (0)

// Device allocation of the runtime (every cudaMalloc of the plans goes through it).
// Host-side fault injection for the error-path tests: with CUNFFT_X_FAULT_ALLOC=k in
// the environment the k-th call in the process (counted from 1) fails as an
// out-of-memory cudaMalloc would, without touching the device; unset, it is cudaMalloc.
cudaError_t plan_malloc(void** ptr, size_t bytes);
template <typename T>
inline cudaError_t plan_malloc(T** ptr, size_t bytes) {
  return plan_malloc(reinterpret_cast<void**>(ptr), bytes);
}
// The same for the cuFFT plan creation: CUNFFT_X_FAULT_CUFFT=k fails the k-th one.
bool plan_fft_fault();

// status helpers
int set_status(Plan* p, int code, const char* fmt, ...);
int check_cuda(Plan* p, cudaError_t e, const char* what);
int check_cufft(Plan* p, cufftResult r, const char* what);

// plan life cycle (plan.cu)
int geom_init(Plan* p, int d, const int64_t* N, const int64_t* n, int m, int prec, int batch);
int plan_init(Plan* p, int d, const int64_t* N, const int64_t* n, int m, int prec, int batch,
              cudaStream_t stream, void* lend_grid);
void plan_release(Plan* p);
int plan_set_nodes(Plan* p, const double* x, const int64_t* M_inst);
int plan_forward(Plan* p, const void* fhat, void* f);
int plan_adjoint(Plan* p, const void* f, void* fhat);
int plan_run_graph(Plan* p, int adjoint, const void* in, void* out);
int plan_interp_only(Plan* p, const void* g, void* f);
int plan_spread_only(Plan* p, const void* f, void* g);
int plan_ndft_forward(Plan* p, const void* fhat, void* f);
int plan_ndft_adjoint(Plan* p, const void* f, void* fhat, const int64_t* kidx = nullptr, int64_t nsel = 0);
int plan_node_gradient(Plan* p, const void* fhat, const void* grad_f, double* grad_x);
// host-buffer transforms with overlapped copies (hostpath.cpp)
int plan_forward_host(Plan* p, const double* x_host, const int64_t* M_inst, const void* fhat_host, void* f_host);
int plan_adjoint_host(Plan* p, const void* f_host, void* fhat_host);
int plan_host_path_sync(Plan* p);
void plan_host_path_release(Plan* p);
int plan_choose_tiling(Plan* p, const int* T, int chunk);
int plan_autotune(Plan* p, int reps);
int plan_set_spread_kernel(Plan* p, int kind);
int plan_spread_kernel(const Plan* p);
int plan_set_interp_kernel(Plan* p, int kind);
int plan_interp_kernel(const Plan* p);

// register-tile spreading kernel (grid_spread_reg.cu)
bool spread_reg_supported(const Plan& p);
size_t spread_reg_smem_bytes(const Plan& p);
cudaError_t grid_launch_spread_reg(const Plan& p, const void* f, void* g, cudaStream_t st);
// tensor-core spreading kernel (grid_spread_tc.cu)
bool spread_tc_supported(const Plan& p);
size_t spread_tc_smem_bytes(const Plan& p);
cudaError_t grid_launch_spread_tc(const Plan& p, const void* f, void* g, cudaStream_t st);
cudaError_t spread_tc_permute(const Plan& p, const void* f, cudaStream_t st);
// failure-reporting check (selftest.cu): a bounded wait that gives up sets *status
cudaError_t launch_wait_gives_up(int32_t* status, cudaStream_t st);
// tensor-core spreading with the A operand in tensor memory (grid_spread_tm.cu); the
// tensor form runs it whenever the tile's planes fit its four M-tiles
bool spread_tm_supported(const Plan& p);
cudaError_t grid_launch_spread_tm(const Plan& p, const void* f, void* g, cudaStream_t st);
// 2D tensor-core spreading kernel (grid_spread2_tm.cu); the tensor form runs it for 2D plans
bool spread2_tm_supported(const Plan& p);
cudaError_t grid_launch_spread2_tm(const Plan& p, const void* f, void* g, cudaStream_t st);
// 2D tensor-core interpolation (grid_interp2_tc.cu): the sub-bins of a tiling it covers
// (16 x 16 sub-tiles of window starts; Tiling::sub_on = 0 where it does not apply)
void interp2_tc_subbins(const Plan& p, Tiling& tl);
// tensor-core interpolation kernel (grid_interp_tc.cu)
bool interp_tc_supported(const Plan& p);
cudaError_t grid_launch_interp_tc(const Plan& p, const void* g, void* f, cudaStream_t st);
cudaError_t interp_tc_prepare(Plan& p);
void interp_tc_release(Plan& p);

// launchers (kernel .cu files); all asynchronous on st
cudaError_t launch_binning(const Plan& p, const double* x, cudaStream_t st);
cudaError_t launch_roc_forward(const Plan& p, const void* fhat, void* g, cudaStream_t st);
cudaError_t launch_roc_adjoint(const Plan& p, const void* g, void* fhat, cudaStream_t st);
cudaError_t launch_interp(const Plan& p, const void* g, void* f, cudaStream_t st);
cudaError_t launch_spread(const Plan& p, const void* f, void* g, cudaStream_t st);
cudaError_t launch_interp_grad(const Plan& p, const void* g, const void* grad_f, double* grad_x, cudaStream_t st);
cudaError_t launch_ndft_forward(const Plan& p, const double* x, const void* fhat, void* f, cudaStream_t st);
cudaError_t launch_ndft_adjoint(const Plan& p, const double* x, const void* f, void* fhat, cudaStream_t st,
                                const int64_t* kidx = nullptr, int64_t nsel = 0);
size_t gridding_smem_bytes(const Plan& p);
int gridding_max_smem(const Plan& p);
bool gridding_supported(int d, int W);

}  // namespace cg
