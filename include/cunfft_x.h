/*
 * cunfft_x.h -- extension API of the GB300 NFFT library (libcunfft.so).
 *
 * New surface beside the drop-in plan API of cunfft.h.  The reference has no
 * counterpart for these entry points except where noted: its plan parameters
 * (m, precision, index width) are compile-time options (src/config.h.in), it
 * runs one transform per plan on the default stream, and its functions return
 * void (src/cunfft.h).  Here:
 *   - m, n and the precision are runtime plan parameters;
 *   - a plan holds B >= 1 instances with uneven node counts M_i (batched form);
 *   - all data pointers are DEVICE pointers (float64 nodes, complex data of the
 *     plan's precision: interleaved double pairs for CUNFFT_X_F64, float pairs
 *     for CUNFFT_X_F32), and every call is asynchronous on the plan's stream;
 *   - every entry point returns a cunfft_x_status code and never exits.
 * Plain C ABI: pointers, sizes and plain integers only.
 */
#ifndef CUNFFT_X_H_
#define CUNFFT_X_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/** Precision of the gridding and FFT stages.  FP64 is the reference's form;
 *  FP32 keeps FP64 only for the node-to-grid reduction and the roll-off factors. */
enum { CUNFFT_X_F64 = 0, CUNFFT_X_F32 = 1 };

/** Spreading (adjoint gridding) kernel.  AUTO picks TENSOR where it applies
 *  (FP32, 2m+2 <= 16, and d = 3 with outer tile extent <= 16 or d = 2 with tile
 *  extents <= 64), else REGISTER (d = 3, FP32, 2m+2 <= 16, outer tile extent <= 8),
 *  else SHARED; GLOBAL is reported when no shared-memory tile fits (wide 3D windows). */
enum {
  CUNFFT_X_SPREAD_AUTO = 0,
  CUNFFT_X_SPREAD_SHARED = 1,   /* padded tile in shared memory, warp-owned planes */
  CUNFFT_X_SPREAD_REGISTER = 2, /* padded tile in registers, one warp per plane */
  CUNFFT_X_SPREAD_GLOBAL = 3,   /* atomics straight into the grid (fallback) */
  CUNFFT_X_SPREAD_TENSOR = 4    /* tile update as FP16 hi/lo x3 tcgen05 MMAs, tile in tensor memory */
};

/** Interpolation (forward gridding) kernel.  AUTO picks TENSOR where it applies
 *  (FP32, 2m+2 <= 16; in 3D an outer tile extent <= 16 and n_3 divisible by 8; in 2D an
 *  inner tile extent >= 16 and n_2 divisible by 8, where the binning orders each tile's
 *  nodes by 16 x 16 sub-tile) and SHARED elsewhere; GLOBAL is reported when no
 *  shared-memory tile fits. */
enum {
  CUNFFT_X_INTERP_AUTO = 0,
  CUNFFT_X_INTERP_SHARED = 1,   /* tile staged in shared memory, warp per node */
  CUNFFT_X_INTERP_GLOBAL = 3,   /* taps read straight from the grid (fallback) */
  CUNFFT_X_INTERP_TENSOR = 4    /* innermost contraction as FP16 hi/lo x3 tcgen05 MMAs */
};

/** Status codes returned by every cunfft_x_* entry point. */
enum cunfft_x_status {
  CUNFFT_X_SUCCESS = 0,
  CUNFFT_X_INVALID_ARGUMENT = 1,
  CUNFFT_X_ALLOC_FAILED = 2,
  CUNFFT_X_CUFFT_ERROR = 3,
  CUNFFT_X_CUDA_ERROR = 4,
  CUNFFT_X_NODES_NOT_SET = 5,
  CUNFFT_X_UNSUPPORTED = 6,
  CUNFFT_X_DEVICE_CHECK_FAILED = 7
};

typedef struct cunfft_x_plan cunfft_x_plan;

/** Create a plan.  d in 1..3; N[d] bandwidths (any N_t >= 1, odd included:
 *  frequencies k_t in [-floor(N_t/2), N_t - floor(N_t/2))); n[d] oversampled grid
 *  sizes, any n_t >= N_t (NULL selects n_t = 2*next_pow2(N_t) like cunfft_init,
 *  src/cunfft.cu:296-299).  The reference wraps window indices with &(n-1)
 *  (src/cunfft_kernel.cu:590, :768, :1036), so there n must be a power of two;
 *  here any size wraps correctly.  The 3D tensor-core gridding forms need an even
 *  last size (spreading) or one divisible by 8 (interpolation), other sizes run the
 *  shared-tile forms; the 2D tensor-core spreading takes any size.  1 <= m <= 15; precision CUNFFT_X_F64 or
 *  CUNFFT_X_F32; batch >= 1 instances; stream 0 creates a private stream
 *  (a cudaStream_t may be passed as void*). */
int cunfft_x_plan_create(cunfft_x_plan **plan, int d, const int64_t *N, const int64_t *n, int m,
                         int precision, int batch, void *stream);

/** Release a plan and its device memory (does not reset the device). */
int cunfft_x_plan_destroy(cunfft_x_plan *plan);

/** Bind a node set: x is a device array of sum_i M_i * d doubles (instance 0's
 *  nodes first, each node's d coordinates contiguous), M_inst a HOST array of
 *  batch node counts.  Bins and sorts the nodes on the device (asynchronous).
 *  The plan keeps the pointer: x must stay valid until the next set_nodes. */
int cunfft_x_set_nodes(cunfft_x_plan *plan, const double *x, const int64_t *M_inst);

/** f = A f_hat for every instance: f_hat has batch*N_total complex values,
 *  f has sum_i M_i (device pointers, plan precision). */
int cunfft_x_forward(cunfft_x_plan *plan, const void *f_hat, void *f);

/** f_hat = A^H f for every instance. */
int cunfft_x_adjoint(cunfft_x_plan *plan, const void *f, void *f_hat);

/** cunfft_x_forward / cunfft_x_adjoint through a CUDA graph.  The first call
 *  for a given (input, output) pair and node binding runs the transform and
 *  captures its stage sequence (roll-off, FFT, gridding of all instances) from
 *  the plan's stream into an instantiated graph; later calls replay it with a
 *  single cudaGraphLaunch.  Binding new nodes or changing the tiling triggers a
 *  new capture.  The plan's stream must be capturable (not the legacy NULL
 *  stream nor a stream that synchronises with it). */
int cunfft_x_forward_graph(cunfft_x_plan *plan, const void *f_hat, void *f);
int cunfft_x_adjoint_graph(cunfft_x_plan *plan, const void *f, void *f_hat);

/** Direct NDFT and adjoint NDFT on the bound nodes, always in FP64 with
 *  complex128 buffers, whatever the plan precision (the error yardstick). */
int cunfft_x_ndft_forward(cunfft_x_plan *plan, const void *f_hat, void *f);
int cunfft_x_ndft_adjoint(cunfft_x_plan *plan, const void *f, void *f_hat);

/** Adjoint NDFT at nsel selected coefficients: kidx is a DEVICE array of
 *  row-major coefficient indices (0 <= kidx < N_total); out receives
 *  batch*nsel complex128 values (instance-major).  For error checks on large
 *  plans where the full adjoint NDFT is out of reach. */
int cunfft_x_ndft_adjoint_at(cunfft_x_plan *plan, const void *f, const int64_t *kidx, int64_t nsel, void *out);

/** Gradient with respect to the node positions of L = sum_j <grad_f_j, f_j>
 *  where f = A(x) f_hat: grad_x[j*d+t] = Re(conj(grad_f_j) * d f_j / d x_{j,t}),
 *  evaluated with the derivative of the Gaussian window on the same grid as the
 *  forward transform.  grad_x is a device array of sum_i M_i * d doubles. */
int cunfft_x_node_gradient(cunfft_x_plan *plan, const void *f_hat, const void *grad_f, double *grad_x);

/** Gridding stages alone, on a caller-provided oversampled grid g
 *  (batch*n_total complex, plan precision): interpolation g -> f and
 *  spreading f -> g (spreading accumulates into g; clear it first).  g needs only
 *  the alignment of its element type (8 bytes for FP32 complex); 16-byte aligned
 *  grids take the wider accesses. */
int cunfft_x_interp(cunfft_x_plan *plan, const void *g, void *f);
int cunfft_x_spread(cunfft_x_plan *plan, const void *f, void *g);

/** Spreading without any memory allocation (no counterpart in the reference).
 *
 *  For callers that cannot allocate device memory: frameworks whose device memory
 *  all belongs to their own pool allocator, real-time loops that must not pay for or
 *  fail on an allocation mid-run, and host applications that forbid allocation in
 *  their plug-in callbacks.  Same result as cunfft_x_spread on a one-instance plan
 *  with these parameters: g += spread of the samples f at the nodes x, where g is
 *  the caller's oversampled grid (prod n complex values of the given precision;
 *  clear it first for a fresh result), x holds M*d doubles and f M complex values,
 *  all device pointers, asynchronous on `stream` (NULL: the legacy default stream).
 *  n may be NULL (n_t = 2*next_pow2(N_t)).  The Gaussian window only.
 *
 *  status: NULL, or a device pointer to one int32 that the call clears on the
 *  stream and that holds, once the spreading has finished, 0 or a non-zero code
 *  when a device-side check failed (a bounded completion wait of the tensor-core
 *  kernel gave up; g is then incomplete).  Read it after synchronising the stream.
 *  With NULL such a failure is not reported.
 *
 *  Its scratch (node bins, tile counts, work queue) is one fixed device array
 *  inside the library, about 58 MB, which every GPU that loads the library holds
 *  until the process exits.  Limits: M <= 1048576 nodes and at most 65536 grid
 *  tiles, the tiles being prod_t ceil(n_t / T_t) for the plan's default tile
 *  extents T.  With m <= 7, 3D tiles are 8 x 8 x 16 (FP32) or 4 x 8 x 16 (FP64), so
 *  n = 256^3 needs 16384 or 32768 tiles and fits, n = 512^3 does not; wider windows
 *  (m >= 8) use 8 x 4 x 8 (FP32) or 4 x 4 x 8 (FP64) tiles in 3D, and a tile whose
 *  padded copy would not fit shared memory is halved along dimension 0.  2D tiles
 *  are 64 x 64 grid points (FP32, m <= 7) or 32 x 64, 1D tiles 2048.
 *  Larger requests return CUNFFT_X_INVALID_ARGUMENT with a message on stderr and
 *  do no device work.  M = 0 leaves g unchanged.
 *
 *  The first call on each device looks up the array's device address
 *  (cudaGetSymbolAddress) and caches it: make that first call before any stream
 *  capture, and do not use the entry point across a device reset.  All calls share
 *  the array: calls that overlap on the GPU (other streams, other host threads on
 *  the same device) race and must be serialised by the caller. */
int cunfft_x_spread_noalloc(int d, const int64_t *N, const int64_t *n, int m, int precision, int64_t M,
                            const double *x, const void *f, void *g, void *stream, int32_t *status);

/** Stream used by the plan (cudaStream_t as void*). */
int cunfft_x_set_stream(cunfft_x_plan *plan, void *stream);
void *cunfft_x_get_stream(const cunfft_x_plan *plan);

/** Tiling of the gridding kernels: tile extents T[d] (powers of two, each
 *  <= n_t) and the maximum number of nodes per work item.  Zeros keep the
 *  defaults.  Re-bins the current node set. */
int cunfft_x_set_tiling(cunfft_x_plan *plan, const int *T, int chunk);

/** Time the candidate tilings on the bound node set and keep the fastest for
 *  spreading and interpolation (reps timed calls per candidate). */
int cunfft_x_autotune(cunfft_x_plan *plan, int reps);

/** Current tiling: T[3], chunk, threads (any pointer may be NULL). */
int cunfft_x_get_tiling(const cunfft_x_plan *plan, int *T, int *chunk, int *threads);

/** Request a spreading kernel (CUNFFT_X_SPREAD_AUTO, _SHARED, _REGISTER or
 *  _TENSOR).  REGISTER or TENSOR on a plan they do not cover returns
 *  CUNFFT_X_UNSUPPORTED and keeps the current kernel.  The request holds across
 *  later tilings (a tiling the requested kernel does not cover runs SHARED). */
int cunfft_x_set_spread_kernel(cunfft_x_plan *plan, int kind);

/** Spreading kernel in use: CUNFFT_X_SPREAD_SHARED, _REGISTER, _TENSOR or _GLOBAL. */
int cunfft_x_get_spread_kernel(const cunfft_x_plan *plan, int *kind);

/** Window of the gridding.  GAUSSIAN is the reference's (src/cunfft.cu:60-87: taps
 *  exp(-(y^2)/b), b = 2 sigma/(2 sigma - 1) m/pi, roll-off exp(pi^2 b k^2/n^2)).
 *  ES is the exponential of semicircle exp(beta (sqrt(1 - y^2/alpha^2) - 1)) on
 *  |y| < alpha = m + 1/2 grid cells, beta = 0.97 pi (2m+1)(1 - 1/(2 sigma))
 *  (Barnett, Magland, af Klinteberg, SIAM J. Sci. Comput. 41 (2019)), roll-off
 *  1/phi_hat(k/n) by Gauss-Legendre quadrature.  Same taps per node (2m+2 per
 *  dimension), same kernels; at sigma = 2 its error falls about tenfold per unit
 *  of window width: about 1e-12 at m = 6 where the Gaussian stops near 1e-6. */
enum {
  CUNFFT_X_WINDOW_GAUSSIAN = 0,
  CUNFFT_X_WINDOW_ES = 1
};

/** Select the window (default GAUSSIAN).  Waits for the plan's stream; bound nodes
 *  stay bound; captured graphs are re-captured on their next launch. */
int cunfft_x_set_window(cunfft_x_plan *plan, int window);

/** Window in use. */
int cunfft_x_get_window(const cunfft_x_plan *plan, int *window);

/** Request an interpolation kernel (CUNFFT_X_INTERP_AUTO, _SHARED or _TENSOR);
 *  TENSOR on a plan it does not cover returns CUNFFT_X_UNSUPPORTED.  The request
 *  holds across later tilings (a tiling TENSOR does not cover runs SHARED). */
int cunfft_x_set_interp_kernel(cunfft_x_plan *plan, int kind);

/** Interpolation kernel in use: CUNFFT_X_INTERP_SHARED, _TENSOR or _GLOBAL. */
int cunfft_x_get_interp_kernel(const cunfft_x_plan *plan, int *kind);

/** Per-stage device times of the last forward/adjoint call, in seconds
 *  (binning, roll-off, FFT, gridding), by stage whatever the direction: after an
 *  adjoint, t_conv is the spreading and t_roc the crop (the reference fills
 *  CUNFFTTimes the same way, src/cunfft.cu:209-224).  Blocks until the plan stream
 *  is idle. */
int cunfft_x_stage_times(cunfft_x_plan *plan, double *t_bin, double *t_roc, double *t_fft, double *t_conv);

/** Forward transform between host buffers, with the copies on the plan's two copy
 *  streams overlapped with its kernels (the reference copies synchronously around
 *  every transform, src/cunfft.cu:107-190).  x_host (sum M[i] x d doubles) with the
 *  per-instance counts M rebinds the nodes first; x_host = NULL keeps the bound
 *  nodes.  fhat_host (batch x N_total complex) in, f_host (sum M complex) out.
 *  Asynchronous: host buffers should be pinned, must stay valid and the inputs
 *  unchanged until cunfft_x_synchronize(plan), which also waits for the copies. */
int cunfft_x_forward_host(cunfft_x_plan *plan, const double *x_host, const int64_t *M, const void *fhat_host,
                          void *f_host);

/** Adjoint between host buffers on the bound nodes: f_host in, fhat_host out; same
 *  rules as cunfft_x_forward_host.  Its upload overlaps a preceding forward. */
int cunfft_x_adjoint_host(cunfft_x_plan *plan, const void *f_host, void *fhat_host);

/** Block until the plan's stream (and the copy streams of the host-buffer
 *  transforms) are idle; reports asynchronous errors and device-side check
 *  failures (CUNFFT_X_DEVICE_CHECK_FAILED, flag cleared on read). */
int cunfft_x_synchronize(cunfft_x_plan *plan);

/** Failure-reporting check.  Launches on the plan's stream a one-thread kernel that
 *  waits, with the bounded mbarrier wait of the tensor-core kernels (here about 1 ms),
 *  on a barrier nothing arrives on; the wait gives up and sets the plan's device
 *  status flag as such a kernel would.  The next cunfft_x_synchronize returns
 *  CUNFFT_X_DEVICE_CHECK_FAILED (and clears the flag); the context stays usable.
 *  Extension (no reference counterpart). */
int cunfft_x_check_wait_timeout(cunfft_x_plan *plan);

/** Last error message of a plan (empty string when none). */
const char *cunfft_x_last_message(const cunfft_x_plan *plan);

/** Human-readable name of a status code. */
const char *cunfft_x_status_string(int status);

/** Oversampled grid of the plan (device pointer; valid until destroy). */
void *cunfft_x_grid(const cunfft_x_plan *plan);

/** Library version string. */
const char *cunfft_x_version(void);

#ifdef __cplusplus
}
#endif

#endif /* CUNFFT_X_H_ */
